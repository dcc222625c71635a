/*
 * swgb_oracle.c -- TEST INFRASTRUCTURE ONLY: the oracle the GB300 kernels are
 * checked against.  It is never linked into, loaded by or called from the
 * swiftshader_gb300 package; only tests/, __graft_entry__.smoke() and
 * bench.py (cpu_baseline leg, --impl reference) use it.
 *
 * A plain-C restatement of google/swiftshader's triangle-list FILL draw path,
 * standalone CMake precision profile (SWIFTSHADER_LEGACY_PRECISION = false,
 * src/Vulkan/VkConfig.hpp:23-24,101-103: 8 sub-pixel bits, fused mulAdd,
 * 16-bit fixed-point filtering of UNORM8 textures).  Each function cites the
 * reference routine it restates.  The reference's JIT code is x86 Reactor;
 * its numeric semantics (src/Reactor/LLVMReactor.cpp) are restated:
 *   - all float math with FTZ+DAZ (worker threads, src/System/SwiftConfig.cpp:136-139),
 *     emulated in software so the oracle gives the same bits on x86 and Arm
 *     (the checker build); the timing build (-DSWGB_ORACLE_HW_FLUSH, used only
 *     to time the CPU baseline) sets the FPU's flush-to-zero mode through
 *     fenv.h on x86-64 and AArch64 instead, as the reference's worker threads
 *     do, and its frames are compared with the checker build's before timing;
 *   - fused multiply-add only where Reactor emits MulAdd/mulAdd;
 *   - RoundInt = cvtss2si/cvtps2dq (half-even, INT_MIN when out of range),
 *     RoundIntClamped = nearbyint + fptosi.sat, Int(Float) = cvttss2si;
 *   - IEEE division for 1/x (Rcp with relaxedPrecision=false on x86,
 *     src/Reactor/Reactor.cpp:4812-4851);
 *   - Max(x, y) = x > y ? x : y, Min(x, y) = x < y ? x : y
 *     (src/Reactor/Reactor.cpp:3980-3988, LLVMReactor.cpp:4443-4453).
 * Build with -fwrapv -ffp-contract=off (int32 wrap-around, no contraction).
 *
 * Unlike the reference it has no OUTLINE_RESOLUTION (8192 rows) limit on the
 * framebuffer height.
 */
#include "swgb_oracle.h"

#include <fenv.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXV 8 /* varying components carried by the fixed shaders */

/* ------------------------------------------------------------------------ */
/* Reactor numeric primitives (a0)                                           */
/* ------------------------------------------------------------------------ */

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* DAZ on inputs / FTZ on results: a subnormal becomes a zero of the same sign. */
#if defined(SWGB_ORACLE_HW_FLUSH) && (defined(__x86_64__) || defined(__aarch64__))
#define ORACLE_HW_FLUSH 1
/* The FPU flushes subnormal inputs and results (hw_flush_on). */
static inline float daz(float x) { return x; }
#else
static inline float daz(float x)
{
    uint32_t u = f2u(x);
    if((u & 0x7F800000u) == 0) return u2f(u & 0x80000000u);
    return x;
}
#endif

/* Timing build: the calling thread's FPU in flush-to-zero mode (MXCSR FTZ +
 * DAZ on x86-64, FPCR.FZ on AArch64), as the reference sets it on its worker
 * threads; new threads inherit it.  The checker build leaves the FPU alone. */
static void hw_flush_on(fenv_t *saved)
{
    fegetenv(saved);
#ifdef ORACLE_HW_FLUSH
    fenv_t e = *saved;
#if defined(__x86_64__)
    e.__mxcsr |= 0x8040u;
#else
    e.__fpcr |= 1u << 24;
#endif
    fesetenv(&e);
#endif
}
static inline float fadd(float a, float b) { return daz(daz(a) + daz(b)); }
static inline float fsub(float a, float b) { return daz(daz(a) - daz(b)); }
static inline float fmul(float a, float b) { return daz(daz(a) * daz(b)); }
static inline float fdiv(float a, float b) { return daz(daz(a) / daz(b)); }
static inline float ffma(float a, float b, float c) { return daz(fmaf(daz(a), daz(b), daz(c))); }

/* Lowering of the mulAdd in QuadRasterizer::interpolate (QuadRasterizer.cpp:235-250,
 * ShaderCore.cpp:714-722): Reactor's LLVM backend emits llvm.fmuladd, fused
 * on an FMA host (the CMake profile this oracle restates, the default);
 * Reactor's Subzero backend emits a multiply and an add
 * (SubzeroReactor.cpp MulAdd).  The routine-level reference fixtures come
 * from a Subzero build, so the tests that compare rasterised depth with them
 * switch this to unfused (oracle_set_interpolation_muladd). */
static int g_interp_fused = 1;
static inline float interp_muladd(float a, float b, float c) { return g_interp_fused ? ffma(a, b, c) : fadd(fmul(a, b), c); }
void oracle_set_interpolation_muladd(int fused) { g_interp_fused = fused != 0; }
/* Comparisons see DAZ-flushed operands. */
static inline int flt(float a, float b) { return daz(a) < daz(b); }
static inline int fle(float a, float b) { return daz(a) <= daz(b); }
static inline int feq(float a, float b) { return daz(a) == daz(b); }
static inline int fgt(float a, float b) { return daz(a) > daz(b); }
static inline float fmaxr(float x, float y) { return fgt(x, y) ? x : y; } /* Max(): x > y ? x : y */
static inline float fminr(float x, float y) { return flt(x, y) ? x : y; } /* Min(): x < y ? x : y */

/* RoundInt (cvtss2si / cvtps2dq; src/Reactor/LLVMReactor.cpp:2373-2381,2684-2692). */
static inline int32_t round_int(float x)
{
    x = daz(x);
    if(!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)nearbyintf(x);
}
/* RoundIntClamped (SIMD::Float; nearbyint + fptosi.sat, LLVMReactor.cpp:4264-4281). */
static inline int32_t round_int_clamped(float x)
{
    x = daz(x);
    if(x != x) return 0;
    float r = nearbyintf(x);
    if(r >= 2147483648.0f) return INT32_MAX;
    if(r < -2147483648.0f) return INT32_MIN;
    return (int32_t)r;
}
/* Int(Float) / Int4(Float4) (cvttss2si / cvttps2dq). */
static inline int32_t trunc_int(float x)
{
    x = daz(x);
    if(!(x >= -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)x;
}
/* MulHigh (pmulhuw / pmulhw; LLVMReactor.cpp:2083-2091,2229-2237). */
static inline uint16_t mulhi_u16(uint16_t a, uint16_t b) { return (uint16_t)(((uint32_t)a * (uint32_t)b) >> 16); }
static inline int16_t mulhi_s16(int16_t a, int16_t b) { return (int16_t)(((int32_t)a * (int32_t)b) >> 16); }
static inline uint16_t addsat_u16(uint16_t a, uint16_t b) { uint32_t s = (uint32_t)a + b; return s > 0xFFFF ? 0xFFFF : (uint16_t)s; }
static inline uint16_t subsat_u16(uint16_t a, uint16_t b) { return a > b ? (uint16_t)(a - b) : 0; }

/* log2sqrt (src/Pipeline/SamplerCore.cpp:1333-1341). */
static float log2sqrt(float lod)
{
    lod = fmul(lod, lod);
    lod = fsub((float)(int32_t)f2u(lod), (float)0x3F800000);
    lod = fmul(lod, u2f(0x33000000));
    return lod;
}

int32_t oracle_round_int(float x) { return round_int(x); }
int32_t oracle_round_int_clamped(float x) { return round_int_clamped(x); }
int32_t oracle_trunc_int(float x) { return trunc_int(x); }
uint16_t oracle_mulhigh_u16(uint16_t a, uint16_t b) { return mulhi_u16(a, b); }
int16_t oracle_mulhigh_s16(int16_t a, int16_t b) { return mulhi_s16(a, b); }
float oracle_fmuladd(float a, float b, float c) { return ffma(a, b, c); }
float oracle_log2sqrt(float x) { return log2sqrt(x); }
float oracle_ftz(float x) { return daz(x); }

/* ------------------------------------------------------------------------ */
/* Draw constants (sw::DrawData, src/Device/Renderer.cpp:300-345)            */
/* ------------------------------------------------------------------------ */

enum { CLIP_RIGHT = 1 << 0, CLIP_TOP = 1 << 1, CLIP_FAR = 1 << 2, CLIP_LEFT = 1 << 3,
       CLIP_BOTTOM = 1 << 4, CLIP_NEAR = 1 << 5, CLIP_FRUSTUM = 0x3F, CLIP_FINITE = 1 << 7 };
/* (src/Device/Clipper.hpp:26-40) */

typedef struct { float x, y, z, w; } f4;

typedef struct {
    f4 pos;          /* clip-space position (Vertex::position)             */
    int clipFlags;
    int X, Y;        /* Vertex::projected.x/y (sub-pixel fixed point)      */
    float pz, pw;    /* Vertex::projected.z/w (z*rhw, rhw)                 */
    float v[MAXV];   /* varyings                                           */
} OVertex;

typedef struct { float A, B, C; } OPlane;

typedef struct {
    const swgb_pipeline_state *st;
    const swgb_draw_args *args;
    float WxF, HxF, X0xF, Y0xF, depthRange, depthNear;
    int sx0, sx1, sy0, sy1;
    int nv;                  /* varying components                       */
    int outCount[SWGB_MAX_ATTRIBS];
    int interpolateZ, interpolateW;
    int depthTest, depthWrite, depthClamp;
    float minDepthClamp, maxDepthClamp;
    int blend;               /* alpha blend active after simplification  */
    uint32_t srcC, dstC, opC, srcA, dstA, opA; /* simplified blend state */
    int rows;                /* span rows per primitive (fb height + 2)  */
    int ms;                  /* samples: 1 or 4                          */
    /* optional visibility record: per sample and pixel, the primitives whose
     * fragment passed the depth test, in primitive order (up to visCap) */
    uint32_t *vis;
    uint32_t *visLen;        /* entries appended (may exceed visCap)      */
    int visCap;
} ODraw;

/* 4x MSAA sample positions (src/Pipeline/Constants.hpp:26-52,
 * src/Pipeline/Constants.cpp:293-294): VkSampleLocations4 relative to the
 * pixel centre (SampleLocationsX/Y) and in sub-pixel fixed point (Xf/Yf). */
static const float SLX[4] = { 0.375f - 0.5f, 0.875f - 0.5f, 0.125f - 0.5f, 0.625f - 0.5f };
static const float SLY[4] = { 0.125f - 0.5f, 0.375f - 0.5f, 0.625f - 0.5f, 0.875f - 0.5f };
static const int XF[4] = { -32, 96, -96, 32 };
static const int YF[4] = { -96, -32, 32, 96 };
#define Y_MIN_MS_OFFSET 159 /* 256 - toFixedPoint(0.375) - 1 */
#define Y_MAX_MS_OFFSET 351 /* 256 + toFixedPoint(0.375) - 1 */

typedef struct {
    int visible;
    uint32_t id;     /* primitive index within the draw */
    int yMin, yMax;
    float x0, y0;
    OPlane z, w, V[MAXV];
    float zBias;     /* Primitive::zBias */
    int front;       /* front-facing: clockwiseMask (SetupRoutine.cpp:104-114) */
    uint16_t *left[4], *right[4]; /* per sample, indexed [y + 1] */
} OPrim;

/* ------------------------------------------------------------------------ */
/* Blend-state simplification (vk::FragmentOutputInterfaceState,             */
/* src/Device/Context.cpp:1090-1270)                                         */
/* ------------------------------------------------------------------------ */

#define OP_ZERO_EXT 1000
#define OP_SRC_EXT 1001
#define OP_DST_EXT 1002

static uint32_t simplify_op(uint32_t op, uint32_t sf, uint32_t df)
{
    switch(op)
    {
    case SWGB_BLEND_OP_ADD:
        if(sf == SWGB_BLEND_ZERO)
        {
            if(df == SWGB_BLEND_ZERO) return OP_ZERO_EXT;
            if(df == SWGB_BLEND_ONE) return OP_DST_EXT;
        }
        else if(sf == SWGB_BLEND_ONE && df == SWGB_BLEND_ZERO)
            return OP_SRC_EXT;
        break;
    case SWGB_BLEND_OP_SUBTRACT:
        if(sf == SWGB_BLEND_ZERO)
        {
            if(df == SWGB_BLEND_ZERO) return OP_ZERO_EXT;
            return OP_ZERO_EXT; /* all attachments here are UNORM or float: UNORM clamps negative to zero */
        }
        else if(sf == SWGB_BLEND_ONE && df == SWGB_BLEND_ZERO)
            return OP_SRC_EXT;
        break;
    case SWGB_BLEND_OP_REVERSE_SUBTRACT:
        if(sf == SWGB_BLEND_ZERO)
        {
            if(df == SWGB_BLEND_ZERO) return OP_ZERO_EXT;
            if(df == SWGB_BLEND_ONE) return OP_DST_EXT;
        }
        break;
    default:
        break;
    }
    return op;
}

/* 8-bit colour attachments: UNORM, or sRGB-encoded UNORM */
static int is_unorm(uint32_t fmt)
{
    return fmt == SWGB_FORMAT_R8G8B8A8_UNORM || fmt == SWGB_FORMAT_B8G8R8A8_UNORM || fmt == SWGB_FORMAT_R8G8B8A8_SRGB ||
           fmt == SWGB_FORMAT_B8G8R8A8_SRGB;
}
static int is_bgra(uint32_t fmt) { return fmt == SWGB_FORMAT_B8G8R8A8_UNORM || fmt == SWGB_FORMAT_B8G8R8A8_SRGB; }
static int is_srgb(uint32_t fmt) { return fmt == SWGB_FORMAT_R8G8B8A8_SRGB || fmt == SWGB_FORMAT_B8G8R8A8_SRGB; }
static int is_tex8(uint32_t fmt)
{
    return fmt == SWGB_FORMAT_R8G8B8A8_UNORM || fmt == SWGB_FORMAT_B8G8R8A8_UNORM || fmt == SWGB_FORMAT_R8G8B8A8_SRGB ||
           fmt == SWGB_FORMAT_B8G8R8A8_SRGB;
}
/* byte of component c (R, G, B, A) in a B8G8R8A8 pixel or texel: R and B swap */
static int bgra_byte(int c) { return c == 0 ? 2 : (c == 2 ? 0 : c); }
static int d16(const swgb_pipeline_state *st) { return st->depth_format == SWGB_FORMAT_D16_UNORM; }

/* sRGBtoLinearFF_FF00 (src/Pipeline/Constants.cpp:273-276), from
 * sw::sRGBtoLinear (src/System/Math.hpp:326-336): 8-bit sRGB to 16-bit linear,
 * 0xFF00 = 1.0. */
static uint16_t srgb_lut[256];
static pthread_once_t srgb_once = PTHREAD_ONCE_INIT;
static void srgb_init(void)
{
    for(int i = 0; i < 256; i++)
    {
        const float c = (float)i / 0xFF;
        const float lin = c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
        srgb_lut[i] = (uint16_t)(lin * 0xFF00 + 0.5f);
    }
}

/* Log2 / Exp2 at relaxed (mediump) precision and Pow<Mediump> = Exp2(Log2(x) * y)
 * (src/Pipeline/ShaderCore.cpp:336-386,406-470,472-477; SWIFTSHADER_LEGACY_PRECISION
 * is false in the CMake build): a bit-pattern log2 with a quadratic mantissa
 * correction; floor/fraction split with a quadratic correction scaled into
 * the exponent field. */
static float log2_mediump(float x)
{
    const int32_t im = (int32_t)f2u(x);
    float y = ffma((float)im, 1.0f / (1 << 23), -127.0f);
    if(im == 0x7F800000) y = u2f(f2u(y) | 0x7F800000u);
    const float m = (float)(im & 0x007FFFFF);
    const float f = ffma(ffma(2.8017103e-22f, m, -8.373131e-15f), m, 5.0615534e-8f);
    return ffma(f, m, y);
}
static float exp2_mediump(float x)
{
    float x0 = fminr(x, 128.0f);
    x0 = fmaxr(x0, u2f(0xC2FDFFFFu));
    const float f = fsub(x0, floorf(daz(x0)));
    const float r = ffma(ffma(7.8145574e-2f, f, 2.2617357e-1f), f, -3.0444314e-1f);
    const float y = ffma(r, f, x0);
    return u2f((uint32_t)trunc_int(ffma((float)(1 << 23), y, (float)(127 << 23))));
}
static float pow_mediump(float x, float y) { return exp2_mediump(fmul(log2_mediump(x), y)); }
/* linearToSRGB / sRGBtoLinear of colour attachments (ShaderCore.cpp:914-930) */
static float linear_to_srgb(float c)
{
    const float lc = fmul(c, 12.92f);
    const float ec = ffma(1.055f, pow_mediump(c, 1.0f / 2.4f), -0.055f);
    return flt(c, 0.0031308f) ? lc : ec;
}
static float srgb_to_linear(float c)
{
    const float lc = fmul(c, 1.0f / 12.92f);
    const float ec = pow_mediump(ffma(c, 1.0f / 1.055f, 0.055f / 1.055f), 2.4f);
    return flt(c, 0.04045f) ? lc : ec;
}
float oracle_linear_to_srgb(float c) { return linear_to_srgb(c); }
float oracle_srgb_to_linear(float c) { return srgb_to_linear(c); }
/* element-wise over arrays, for the known-answer and error-bound tests:
 * fn 0 Log2 mediump, 1 Exp2 mediump, 2 linearToSRGB, 3 sRGBtoLinear */
void oracle_transcendental_n(int fn, const float *in, float *out, size_t n)
{
    for(size_t i = 0; i < n; i++)
        out[i] = fn == 0 ? log2_mediump(in[i]) : fn == 1 ? exp2_mediump(in[i]) : fn == 2 ? linear_to_srgb(in[i]) : srgb_to_linear(in[i]);
}

/* ------------------------------------------------------------------------ */
/* Validation + DrawData                                                     */
/* ------------------------------------------------------------------------ */

static swgb_status prepare(ODraw *d, const swgb_pipeline_state *st, const swgb_draw_args *a)
{
    memset(d, 0, sizeof(*d));
    d->st = st;
    d->args = a;
    if(st->precision_profile != SWGB_PRECISION_CMAKE) return SWGB_UNSUPPORTED_STATE;
    if(st->topology != SWGB_TOPOLOGY_TRIANGLE_LIST && st->topology != SWGB_TOPOLOGY_TRIANGLE_STRIP &&
       st->topology != SWGB_TOPOLOGY_TRIANGLE_FAN)
        return SWGB_UNSUPPORTED_STATE;
    if(st->sample_count != 1 && st->sample_count != 4) return SWGB_UNSUPPORTED_STATE;
    if(st->depth_clamp_enable) return SWGB_UNSUPPORTED_STATE;
    if(st->attrib_count < 1 || st->attrib_count > SWGB_MAX_ATTRIBS) return SWGB_INVALID_ARG;
    if(!is_unorm(st->color_format) && st->color_format != SWGB_FORMAT_R32G32B32A32_SFLOAT &&
       st->color_format != SWGB_FORMAT_R16G16B16A16_SFLOAT)
        return SWGB_UNSUPPORTED_STATE;
    if(st->fragment_shader == SWGB_FS_TEX_X_VCOLOR && !is_tex8(st->texture.format) &&
       st->texture.format != SWGB_FORMAT_R16G16B16A16_SFLOAT && st->texture.format != SWGB_FORMAT_R32G32B32A32_SFLOAT)
        return SWGB_UNSUPPORTED_STATE;
    if(st->depth_format != SWGB_FORMAT_UNDEFINED && st->depth_format != SWGB_FORMAT_D32_SFLOAT && st->depth_format != SWGB_FORMAT_D16_UNORM)
        return SWGB_UNSUPPORTED_STATE;
    pthread_once(&srgb_once, srgb_init);

    /* Viewport (Renderer.cpp:300-331) */
    float W = 0.5f * st->viewport_width;
    float H = 0.5f * st->viewport_height;
    float X0 = st->viewport_x + W;
    float Y0 = st->viewport_y + H;
    float N = st->viewport_min_depth;
    float F = st->viewport_max_depth;
    const float subPixF = 256.0f;
    d->WxF = W * subPixF;
    d->HxF = H * subPixF;
    d->X0xF = X0 * subPixF - subPixF / 2;
    d->Y0xF = Y0 * subPixF - subPixF / 2;
    d->depthRange = F - N;
    d->depthNear = N;

    /* Scissor (Renderer.cpp:333-345) */
    int x0 = a->render_area_x, y0 = a->render_area_y;
    int x1 = x0 + (int)a->render_area_width, y1 = y0 + (int)a->render_area_height;
#define CLAMPI(v, lo, hi) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
    d->sx0 = CLAMPI(st->scissor_x, x0, x1);
    d->sx1 = CLAMPI(st->scissor_x + (int)st->scissor_width, x0, x1);
    d->sy0 = CLAMPI(st->scissor_y, y0, y1);
    d->sy1 = CLAMPI(st->scissor_y + (int)st->scissor_height, y0, y1);
    if(d->sx1 > (int)st->framebuffer_width || d->sy1 > (int)st->framebuffer_height || d->sx0 < 0 || d->sy0 < 0)
        return SWGB_INVALID_ARG;

    /* Varyings of the fixed VS: location k = attribute k+1. */
    d->nv = 0;
    for(uint32_t i = 1; i < st->attrib_count; i++)
    {
        int c = st->attribs[i].format == SWGB_FORMAT_R32G32_SFLOAT ? 2 : 4;
        d->outCount[i] = c;
        d->nv += c;
    }
    if(d->nv > MAXV) return SWGB_UNSUPPORTED_STATE;
    if(st->fragment_shader == SWGB_FS_VCOLOR && (st->attrib_count < 2 || d->outCount[1] != 4)) return SWGB_INVALID_ARG;
    if(st->fragment_shader == SWGB_FS_TEX_X_VCOLOR && (st->attrib_count < 3 || d->outCount[1] != 4)) return SWGB_INVALID_ARG;

    /* SetupProcessor::update (src/Device/SetupProcessor.cpp:58-103) */
    d->depthTest = st->depth != NULL && st->depth_test_enable;
    d->depthWrite = d->depthTest && st->depth_write_enable;
    d->interpolateZ = d->depthTest;
    d->interpolateW = 1; /* a fragment shader is always present */
    /* PixelProcessor::update depth clamp (src/Device/PixelProcessor.cpp:106-128):
     * without VK_EXT_depth_range_unrestricted depth is clamped to [0,1]. */
    d->depthClamp = 1;
    d->minDepthClamp = 0.0f;
    d->maxDepthClamp = 1.0f;

    /* Blend (Context.cpp:1090-1160) */
    uint32_t opC = simplify_op(st->color_blend_op, st->src_color_factor, st->dst_color_factor);
    uint32_t opA = simplify_op(st->alpha_blend_op, st->src_alpha_factor, st->dst_alpha_factor);
    d->blend = st->blend_enable && (opC != OP_SRC_EXT || opA != OP_SRC_EXT) && st->color_write_mask != 0;
    d->srcC = st->src_color_factor; d->dstC = st->dst_color_factor; d->opC = opC;
    d->srcA = st->src_alpha_factor; d->dstA = st->dst_alpha_factor; d->opA = opA;
    if(st->color_blend_op > SWGB_BLEND_OP_MAX || st->alpha_blend_op > SWGB_BLEND_OP_MAX) return SWGB_UNSUPPORTED_STATE;

    d->rows = (int)st->framebuffer_height + 2;
    d->ms = (int)st->sample_count;
    return SWGB_OK;
}

/* ------------------------------------------------------------------------ */
/* Vertex stage (src/Pipeline/VertexRoutine.cpp, VertexProgram.cpp)          */
/* ------------------------------------------------------------------------ */

static uint32_t vertex_index(const ODraw *d, uint32_t k)
{
    const swgb_draw_args *a = d->args;
    uint32_t idx;
    if(a->index_type == SWGB_INDEX_TYPE_NONE)
        idx = a->first_vertex + k;
    else if(a->index_type == SWGB_INDEX_TYPE_UINT16)
        idx = ((const uint16_t *)a->indices)[k];
    else if(a->index_type == SWGB_INDEX_TYPE_UINT8)
        idx = ((const uint8_t *)a->indices)[k];
    else
        idx = ((const uint32_t *)a->indices)[k];
    return idx + (uint32_t)a->base_vertex; /* readStream: (index + baseVertex) * stride, UInt arithmetic */
}

static void read_attrib(const ODraw *d, int i, uint32_t index, float out[4])
{
    const swgb_vertex_attrib *at = &d->st->attribs[i];
    const swgb_vertex_binding *b = &d->st->bindings[at->binding];
    const uint8_t *p = (const uint8_t *)b->buffer + (size_t)index * b->stride + at->offset;
    if(at->format == SWGB_FORMAT_R32G32_SFLOAT)
    {
        memcpy(out, p, 8);
        out[2] = 0.0f;
        out[3] = 1.0f; /* readStream: componentCount < 4 -> w = 1 (VertexRoutine.cpp:565) */
    }
    else
        memcpy(out, p, 16);
}

static void vertex_shade(const ODraw *d, uint32_t index, OVertex *o)
{
    const swgb_pipeline_state *st = d->st;
    float p[4];
    read_attrib(d, 0, index, p);
    /* OpMatrixTimesVector (SpirvShaderArithmetic.cpp:39-55): v = m[0][i]*p0, then
     * MulAdd(m[j][i], p_j, v) for j = 1..3; the matrix is column-major. */
    float r[4];
    for(int i = 0; i < 4; i++)
    {
        float v = fmul(st->mvp[0 * 4 + i], p[0]);
        for(int j = 1; j < 4; j++) v = ffma(st->mvp[j * 4 + i], p[j], v);
        r[i] = v;
    }
    o->pos.x = r[0]; o->pos.y = r[1]; o->pos.z = r[2]; o->pos.w = r[3];

    /* computeClipFlags (VertexRoutine.cpp:116-154) */
    float x = r[0], y = r[1], z = r[2], w = r[3];
    int f = 0;
    if(flt(w, x)) f |= CLIP_RIGHT;
    if(flt(w, y)) f |= CLIP_TOP;
    if(!fle(-w, x)) f |= CLIP_LEFT;
    if(!fle(-w, y)) f |= CLIP_BOTTOM;
    if(st->depth_clip_enable)
    {
        if(flt(w, z)) f |= CLIP_FAR;
        if(!fle(0.0f, z)) f |= CLIP_NEAR;
    }
    const float maxPos = u2f(0x7F7FFFFF);
    if(fle(fabsf(x), maxPos) && fle(fabsf(y), maxPos) && fle(fabsf(z), maxPos)) f |= CLIP_FINITE;
    o->clipFlags = f;

    /* writeCache projection (VertexRoutine.cpp:599-612) */
    uint32_t wb = f2u(w);
    if(feq(w, 0.0f)) wb |= f2u(1.0f);
    float ww = u2f(wb);
    float rhw = fdiv(1.0f, ww);
    o->X = round_int_clamped(fadd(d->X0xF, fmul(fmul(x, rhw), d->WxF)));
    o->Y = round_int_clamped(fadd(d->Y0xF, fmul(fmul(y, rhw), d->HxF)));
    o->pz = fmul(z, rhw);
    o->pw = rhw;

    /* pass-through varyings */
    int k = 0;
    for(uint32_t i = 1; i < st->attrib_count; i++)
    {
        float a[4];
        read_attrib(d, (int)i, index, a);
        for(int c = 0; c < d->outCount[i]; c++) o->v[k++] = a[c];
    }
}

/* ------------------------------------------------------------------------ */
/* Clipper (src/Device/Clipper.cpp:22-299)                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    f4 B[16];
    const f4 *P[16][16];
    int n, i, b;
} OPolygon;

static void clip_edge(f4 *Vo, const f4 *Vi, const f4 *Vj, float di, float dj)
{
    float D = fdiv(1.0f, fsub(dj, di));
    Vo->x = fmul(fsub(fmul(dj, Vi->x), fmul(di, Vj->x)), D);
    Vo->y = fmul(fsub(fmul(dj, Vi->y), fmul(di, Vj->y)), D);
    Vo->z = fmul(fsub(fmul(dj, Vi->z), fmul(di, Vj->z)), D);
    Vo->w = fmul(fsub(fmul(dj, Vi->w), fmul(di, Vj->w)), D);
}

/* plane: 0 near(z), 1 far(w-z), 2 left(w+x), 3 right(w-x), 4 top(w-y), 5 bottom(w+y) */
static float plane_dist(const f4 *v, int plane)
{
    switch(plane)
    {
    case 0: return v->z;
    case 1: return fsub(v->w, v->z);
    case 2: return fadd(v->w, v->x);
    case 3: return fsub(v->w, v->x);
    case 4: return fsub(v->w, v->y);
    default: return fadd(v->w, v->y);
    }
}

static void clip_plane(OPolygon *p, int plane)
{
    const f4 **V = p->P[p->i];
    const f4 **T = p->P[p->i + 1];
    int t = 0;
    for(int i = 0; i < p->n; i++)
    {
        int j = i == p->n - 1 ? 0 : i + 1;
        float di = plane_dist(V[i], plane);
        float dj = plane_dist(V[j], plane);
        if(fle(0.0f, di)) /* di >= 0 */
        {
            T[t++] = V[i];
            if(flt(dj, 0.0f))
            {
                clip_edge(&p->B[p->b], V[i], V[j], di, dj);
                T[t++] = &p->B[p->b++];
            }
        }
        else
        {
            if(fgt(dj, 0.0f))
            {
                clip_edge(&p->B[p->b], V[j], V[i], dj, di);
                T[t++] = &p->B[p->b++];
            }
        }
    }
    p->n = t;
    p->i += 1;
}

static int clip_polygon(OPolygon *p, int flagsOr)
{
    static const int order[6] = { CLIP_NEAR, CLIP_FAR, CLIP_LEFT, CLIP_RIGHT, CLIP_TOP, CLIP_BOTTOM };
    if(flagsOr & CLIP_FRUSTUM)
    {
        for(int k = 0; k < 6; k++)
        {
            if(p->n < 3) break;
            if(flagsOr & order[k]) clip_plane(p, k);
        }
    }
    return p->n >= 3;
}

/* ------------------------------------------------------------------------ */
/* Setup (src/Pipeline/SetupRoutine.cpp:36-621)                              */
/* ------------------------------------------------------------------------ */

static inline int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return x < lo ? lo : (x > hi ? hi : x); }
static inline int32_t shl(int32_t x, int s) { return (int32_t)((uint32_t)x << s); }

/* SetupRoutine::edge (SetupRoutine.cpp:550-621) */
static void setup_edge(const ODraw *d, OPrim *pr, int q, int32_t Xa, int32_t Ya, int32_t Xb, int32_t Yb)
{
    if(Ya == Yb) return;
    int swap = Yb < Ya;
    int32_t X1 = swap ? Xb : Xa, X2 = swap ? Xa : Xb;
    int32_t Y1 = swap ? Yb : Ya, Y2 = swap ? Ya : Yb;
    int32_t y1 = (Y1 + 0xFF) >> 8;
    int32_t y2 = (Y2 + 0xFF) >> 8;
    int32_t yMin = y1 > d->sy0 ? y1 : d->sy0;
    int32_t yMax = y2 < d->sy1 ? y2 : d->sy1;
    if(!(yMin < yMax)) return;
    uint16_t *edge = swap ? pr->right[q] : pr->left[q];
    int32_t DX12 = X2 - X1, DY12 = Y2 - Y1;
    int32_t FDX12 = shl(DX12, 8), FDY12 = shl(DY12, 8);
    int32_t X = DX12 * (shl(y1, 8) - Y1) + (X1 & 0xFF) * DY12;
    int32_t x = (X1 >> 8) + X / FDY12;
    int32_t dd = X % FDY12;
    int32_t ceil_ = (-dd) >> 31;
    x -= ceil_;
    dd -= ceil_ & FDY12;
    int32_t Q = FDX12 / FDY12, R = FDX12 % FDY12;
    int32_t floor_ = R >> 31;
    Q += floor_;
    R += floor_ & FDY12;
    int32_t D = FDY12;
    int32_t y = y1;
    do
    {
        if(y >= yMin) edge[y + 1] = (uint16_t)clampi(x, d->sx0, d->sx1);
        x += Q;
        dd += R;
        int32_t overflow = (-dd) >> 31;
        dd -= D & overflow;
        x -= overflow;
        y++;
    } while(y < yMax);
}

static void set_vertices(const OVertex *v0, const OVertex *v1, const OVertex *v2, const OVertex **out)
{
    out[0] = v0; out[1] = v1; out[2] = v2;
}

/* SetupRoutine::generate for a solid triangle (SetupRoutine.cpp:36-512).
 * 'poly' is the (possibly clipped) polygon; returns 1 if visible. */
static int setup_triangle(const ODraw *d, const OVertex *tv0, const OVertex *tv1, const OVertex *tv2, const OPolygon *poly, OPrim *pr)
{
    const swgb_pipeline_state *st = d->st;
    int32_t X[17], Y[17];
    X[0] = tv0->X; X[1] = tv1->X; X[2] = tv2->X;
    Y[0] = tv0->Y; Y[1] = tv1->Y; Y[2] = tv2->Y;
    int dW = 1;

    /* Culling (:73-120) */
    {
        float x0 = (float)X[0], x1 = (float)X[1], x2 = (float)X[2];
        float y0 = (float)Y[0], y1 = (float)Y[1], y2 = (float)Y[2];
        float A = fadd(fadd(fmul(fsub(y0, y2), x1), fmul(fsub(y2, y1), x0)), fmul(fsub(y1, y0), x2));
        int32_t w0w1w2 = (int32_t)(f2u(tv0->pos.w) ^ f2u(tv1->pos.w) ^ f2u(tv2->pos.w));
        if(w0w1w2 < 0) A = -A;
        int frontFacing = st->front_face == SWGB_FRONT_FACE_COUNTER_CLOCKWISE ? fle(0.0f, A) : fle(A, 0.0f);
        if((st->cull_mode & SWGB_CULL_FRONT) && frontFacing) return 0;
        if((st->cull_mode & SWGB_CULL_BACK) && !frontFacing) return 0;
        dW = fgt(A, 0.0f) ? 1 : 0;
        pr->front = frontFacing;
    }

    int n = poly->n;
    int m = poly->i;
    if(m != 0) /* clipped triangle; reproject (:125-145) */
    {
        for(int i = 0; i < n; i++)
        {
            const f4 *p = poly->P[m][i];
            float w = p->w;
            float rhw = !feq(w, 0.0f) ? fdiv(1.0f, w) : 1.0f;
            X[i] = round_int(fadd(d->X0xF, fmul(fmul(p->x, rhw), d->WxF)));
            Y[i] = round_int(fadd(d->Y0xF, fmul(fmul(p->y, rhw), d->HxF)));
        }
    }

    /* Vertical range (:147-186) */
    int32_t yMin = Y[0], yMax = Y[0];
    for(int i = 1; i < n; i++)
    {
        yMin = Y[i] < yMin ? Y[i] : yMin;
        yMax = Y[i] > yMax ? Y[i] : yMax;
    }
    if(d->ms > 1)
    {
        yMin = (yMin + Y_MIN_MS_OFFSET) >> 8;
        yMax = (yMax + Y_MAX_MS_OFFSET) >> 8;
    }
    else
    {
        yMin = (yMin + 0xFF) >> 8;
        yMax = (yMax + 0xFF) >> 8;
    }
    yMin = yMin > d->sy0 ? yMin : d->sy0;
    yMax = yMax < d->sy1 ? yMax : d->sy1;
    if(yMin >= yMax) return 0;

    /* Rasterize the outline of every sample (:188-240) */
    for(int q = 0; q < d->ms; q++)
    {
        int32_t Xq[17], Yq[17];
        for(int i = 0; i < n; i++)
        {
            Xq[i] = X[i];
            Yq[i] = Y[i];
            if(d->ms > 1)
            {
                /* the edge is tested against the sample point (:199-203) */
                Xq[i] = Xq[i] - XF[q];
                Yq[i] = Yq[i] - YF[q];
            }
        }
        if(d->ms > 1)
        {
            int32_t x = clampi((X[0] + 0xFF) >> 8, d->sx0, d->sx1);
            for(int32_t y = yMin - 1; y < yMax + 1; y++)
            {
                pr->left[q][y + 1] = (uint16_t)x;
                pr->right[q][y + 1] = (uint16_t)x;
            }
        }
        Xq[n] = Xq[0];
        Yq[n] = Yq[0];
        for(int i = 0; i < n; i++)
            setup_edge(d, pr, q, Xq[i + 1 - dW], Yq[i + 1 - dW], Xq[i + dW], Yq[i + dW]);
        if(d->ms == 1)
        {
            /* Trim empty rows and pad (:243-264) */
            uint16_t *L = pr->left[0], *R = pr->right[0];
            while(yMin < yMax && L[yMin + 1] == R[yMin + 1]) yMin++;
            while(yMax > yMin && L[yMax - 1 + 1] == R[yMax - 1 + 1]) yMax--;
            if(yMin == yMax) return 0;
            L[yMin - 1 + 1] = L[yMin + 1];
            R[yMin - 1 + 1] = L[yMin + 1];
            L[yMax + 1] = L[yMax - 1 + 1];
            R[yMax + 1] = L[yMax - 1 + 1];
        }
    }
    pr->yMin = yMin;
    pr->yMax = yMax;

    /* Sort by minimum y, then maximum w (:270-294) */
    const OVertex *v[3];
    set_vertices(tv0, tv1, tv2, v);
    {
        float y0 = v[0]->pos.y, y1 = v[1]->pos.y, y2 = v[2]->pos.y;
        float ym = fminr(fminr(y0, y1), y2);
        const OVertex *t;
        if(feq(ym, y1)) { t = v[0]; v[0] = v[1]; v[1] = v[2]; v[2] = t; }
        if(feq(ym, y2)) { t = v[2]; v[2] = v[1]; v[1] = v[0]; v[0] = t; }
    }
    {
        float w0 = v[0]->pos.w, w1 = v[1]->pos.w, w2 = v[2]->pos.w;
        float wm = fmaxr(fmaxr(w0, w1), w2);
        const OVertex *t;
        if(feq(wm, w1)) { t = v[0]; v[0] = v[1]; v[1] = v[2]; v[2] = t; }
        if(feq(wm, w2)) { t = v[2]; v[2] = v[1]; v[1] = v[0]; v[0] = t; }
    }

    /* Plane equations (:296-415) */
    float w1 = v[1]->pos.w, w2 = v[2]->pos.w; /* w0 only feeds noperspective varyings */
    float rhw0 = v[0]->pw;
    int32_t X0 = v[0]->X, X1 = v[1]->X, X2 = v[2]->X;
    int32_t Y0 = v[0]->Y, Y1 = v[1]->Y, Y2 = v[2]->Y;
    const float inv = 1.0f / 256.0f;
    pr->x0 = fmul((float)X0, inv);
    pr->y0 = fmul((float)Y0, inv);
    X1 -= X0; Y1 -= Y0;
    X2 -= X0; Y2 -= Y0;
    float x1 = fmul(fmul(w1, inv), (float)X1);
    float y1 = fmul(fmul(w1, inv), (float)Y1);
    float x2 = fmul(fmul(w2, inv), (float)X2);
    float y2 = fmul(fmul(w2, inv), (float)Y2);
    float a = fsub(fmul(x1, y2), fmul(x2, y1));
    f4 M[3];
    memset(M, 0, sizeof(M));
    M[0].z = rhw0;
    if(!feq(a, 0.0f))
    {
        float A = fdiv(1.0f, a);
        float D = fmul(A, rhw0);
        M[0].x = fmul(fsub(fmul(y1, w2), fmul(y2, w1)), D);
        M[0].y = fmul(fsub(fmul(x2, w1), fmul(x1, w2)), D);
        M[1].x = fmul(y2, A);
        M[1].y = fmul(-x2, A);
        M[2].x = fmul(-y1, A);
        M[2].y = fmul(x1, A);
    }
    if(d->interpolateW)
    {
        pr->w.A = fadd(fadd(M[0].x, M[1].x), M[2].x);
        pr->w.B = fadd(fadd(M[0].y, M[1].y), M[2].y);
        pr->w.C = fadd(fadd(M[0].z, M[1].z), M[2].z);
    }
    if(d->interpolateZ)
    {
        float z0 = v[0]->pz, z1 = v[1]->pz, z2 = v[2]->pz;
        z1 = fsub(z1, z0);
        z2 = fsub(z2, z0);
        float fx1 = fmul((float)X1, inv), fy1 = fmul((float)Y1, inv);
        float fx2 = fmul((float)X2, inv), fy2 = fmul((float)Y2, inv);
        float D = fdiv(d->depthRange, fsub(fmul(fx1, fy2), fmul(fx2, fy1)));
        pr->z.A = fmul(fsub(fmul(fy2, z1), fmul(fy1, z2)), D);
        pr->z.B = fmul(fsub(fmul(fx1, z2), fmul(fx2, z1)), D);
        pr->z.C = fadd(fmul(z0, d->depthRange), d->depthNear);
        /* depth bias (:417-476) */
        const swgb_pipeline_state *st = d->st;
        pr->zBias = 0.0f;
        if(st->depth_bias_constant != 0.0f || st->depth_bias_slope != 0.0f)
        {
            float bias = 0.0f;
            if(st->depth_bias_constant != 0.0f)
            {
                float r; /* minimum resolvable difference */
                if(d16(st)) r = 1.01f / 0xFFFF; /* Renderer.cpp:426-430 */
                else
                {
                    /* 2^(e-23), e the largest exponent of Z0, Z1, Z2; Z1 and Z2
                     * are formed from the differences z1, z2 as the reference does */
                    float Z0 = pr->z.C;
                    float Z1 = fadd(fmul(z1, d->depthRange), d->depthNear);
                    float Z2 = fadd(fmul(z2, d->depthRange), d->depthNear);
                    int32_t e0 = (int32_t)(f2u(Z0) & 0x7F800000u), e1 = (int32_t)(f2u(Z1) & 0x7F800000u), e2 = (int32_t)(f2u(Z2) & 0x7F800000u);
                    int32_t e = e0 > e1 ? e0 : e1;
                    e = e > e2 ? e : e2;
                    r = fmul(u2f((uint32_t)e), 1.0f / (1 << 23));
                }
                bias = fmul(r, st->depth_bias_constant);
            }
            if(st->depth_bias_slope != 0.0f)
            {
                float m = fmaxr(fabsf(pr->z.A), fabsf(pr->z.B));
                bias = fadd(bias, fmul(m, st->depth_bias_slope));
            }
            float clamp = st->depth_bias_clamp == st->depth_bias_clamp ? st->depth_bias_clamp : 0.0f; /* Context.cpp:650-661 */
            if(clamp != 0.0f) bias = clamp > 0.0f ? fminr(bias, clamp) : fmaxr(bias, clamp);
            pr->zBias = bias;
        }
    }
    /* setupGradient, smooth (perspective) varyings (:478-548) */
    for(int k = 0; k < d->nv; k++)
    {
        float i0 = v[0]->v[k], i1 = v[1]->v[k], i2 = v[2]->v[k];
        pr->V[k].A = fadd(fadd(fmul(i0, M[0].x), fmul(i1, M[1].x)), fmul(i2, M[2].x));
        pr->V[k].B = fadd(fadd(fmul(i0, M[0].y), fmul(i1, M[1].y)), fmul(i2, M[2].y));
        pr->V[k].C = fadd(fadd(fmul(i0, M[0].z), fmul(i1, M[1].z)), fmul(i2, M[2].z));
    }
    return 1;
}

/* setupSolidTriangles for one triangle (src/Device/Renderer.cpp:733-776).
 * Returns visibility; counters updated. */
/* Index-buffer positions of triangle tri: setBatchIndices
 * (src/Device/Renderer.cpp:49-145), provokeFirst = provoking vertex FIRST. */
static void triangle_positions(uint32_t topology, int provokeFirst, uint32_t tri, uint32_t k[3])
{
    switch(topology)
    {
    case SWGB_TOPOLOGY_TRIANGLE_STRIP: /* :110-121 */
        k[0] = tri + (provokeFirst ? 0 : 2);
        k[1] = tri + (tri & 1) + (provokeFirst ? 1 : 0);
        k[2] = tri + (~tri & 1) + (provokeFirst ? 1 : 0);
        break;
    case SWGB_TOPOLOGY_TRIANGLE_FAN: /* :122-133: index = tri + 1 */
        k[provokeFirst ? 0 : 2] = tri + 1;
        k[provokeFirst ? 1 : 0] = tri + 2;
        k[provokeFirst ? 2 : 1] = 0;
        break;
    default: /* TRIANGLE_LIST :97-109 */
        k[0] = 3 * tri + (provokeFirst ? 0 : 2);
        k[1] = 3 * tri + (provokeFirst ? 1 : 0);
        k[2] = 3 * tri + (provokeFirst ? 2 : 1);
        break;
    }
}

static int process_triangle(const ODraw *d, uint32_t tri, OPrim *pr, swgb_counters *cnt, int *clipped_out)
{
    OVertex v0, v1, v2;
    uint32_t k[3];
    triangle_positions(d->st->topology, d->st->provoking_vertex == 0, tri, k);
    vertex_shade(d, vertex_index(d, k[0]), &v0);
    vertex_shade(d, vertex_index(d, k[1]), &v1);
    vertex_shade(d, vertex_index(d, k[2]), &v2);
    OPolygon poly;
    poly.P[0][0] = &v0.pos; poly.P[0][1] = &v1.pos; poly.P[0][2] = &v2.pos;
    poly.n = 3; poly.i = 0; poly.b = 0;
    *clipped_out = 0;
    pr->visible = 0;
    /* cullMask is 0xF for every vertex: the fixed VS writes no cull distances */
    if((v0.clipFlags & v1.clipFlags & v2.clipFlags) != CLIP_FINITE) return 0;
    int flagsOr = v0.clipFlags | v1.clipFlags | v2.clipFlags;
    if(flagsOr != CLIP_FINITE)
    {
        *clipped_out = 1;
        if(!clip_polygon(&poly, flagsOr)) return 0;
    }
    pr->visible = setup_triangle(d, &v0, &v1, &v2, &poly, pr);
    (void)cnt;
    return pr->visible;
}

/* ------------------------------------------------------------------------ */
/* SamplerCore, 16-bit fixed-point path for R8G8B8A8_UNORM                   */
/* (src/Pipeline/SamplerCore.cpp)                                            */
/* ------------------------------------------------------------------------ */

typedef struct {
    const swgb_texture *t;
    float W, H;        /* Texture::widthWidthHeightHeight (level 0)   */
    float minLod, maxLod, bias;
    int linearFilter;  /* FILTER_LINEAR vs FILTER_POINT               */
    int mipLinear;     /* MIPMAP_LINEAR vs MIPMAP_POINT               */
} OSampler;

static void sampler_init(OSampler *s, const swgb_texture *t)
{
    s->t = t;
    s->W = (float)t->levels[0].width;
    s->H = (float)t->levels[0].height;
    s->bias = t->mip_lod_bias;
    /* vk::Sampler ClampLod (src/Vulkan/VkSampler.hpp:33-36) */
    float mn = t->min_lod, mx = t->max_lod;
    mn = mn < 0.0f ? 0.0f : (mn > 13.0f ? 13.0f : mn);
    mx = mx < 0.0f ? 0.0f : (mx > 13.0f ? 13.0f : mx);
    /* FILTER_* (SpirvShaderSampling.cpp:275-326); mixed min/mag filters unsupported. */
    s->linearFilter = t->mag_filter == SWGB_FILTER_LINEAR;
    s->mipLinear = t->mipmap_mode == SWGB_MIPMAP_MODE_LINEAR;
    /* single mip level forces minLod = maxLod = 0 (SpirvShaderSampling.cpp:88-99) */
    if(t->level_count == 1) { mn = 0.0f; mx = 0.0f; }
    s->minLod = mn;
    s->maxLod = mx;
}

static const swgb_texture_level *level_at(const OSampler *s, int index)
{
    /* Descriptor replicates the last level (VkDescriptorSetLayout.cpp:468-470). */
    int l = index < 0 ? 0 : index;
    if(l > (int)s->t->level_count - 1) l = (int)s->t->level_count - 1;
    return &s->t->levels[l];
}

/* address() 16-bit (SamplerCore.cpp:2399-2435) */
static uint16_t address16(float uw, uint32_t mode)
{
    if(mode == SWGB_ADDRESS_CLAMP_TO_EDGE)
    {
        float c = fminr(fmaxr(uw, 0.0f), 65535.0f / 65536.0f);
        return (uint16_t)trunc_int(fmul(c, 65536.0f));
    }
    if(mode == SWGB_ADDRESS_MIRRORED_REPEAT)
    {
        int32_t convert = trunc_int(fmul(uw, 65536.0f));
        int32_t mirror = shl(convert, 15) >> 31;
        convert ^= mirror;
        return (uint16_t)convert;
    }
    if(mode == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE)
    {
        /* ADDRESSING_MIRRORONCE: Int4(Abs(u * 2^16)) - 0x8000 (wrapping int32),
         * PackSigned to int16, + 0x8000 as uint16 */
        int32_t convert = (int32_t)((uint32_t)trunc_int(fabsf(fmul(uw, 65536.0f))) - 0x8000u);
        convert = convert < -32768 ? -32768 : (convert > 32767 ? 32767 : convert);
        return (uint16_t)(convert + 0x8000);
    }
    return (uint16_t)trunc_int(fmul(uw, 65536.0f)); /* wrap */
}

/* offsetSample (SamplerCore.cpp:278-313) */
static uint16_t offset_sample(uint16_t uvw, uint16_t half, int wrap, int count)
{
    if(wrap) return count < 0 ? (uint16_t)(uvw - half) : (uint16_t)(uvw + half);
    return count < 0 ? subsat_u16(uvw, half) : addsat_u16(uvw, half);
}

/* computeIndices + sampleTexel for 8-bit RGBA textures (SamplerCore.cpp:
 * 1593-1643,1747-1788): texel component c is returned as c << 8; B8G8R8A8
 * texels swap R and B; the R, G, B of sRGB textures are replaced by their
 * sRGBtoLinearFF_FF00 entry (:1966-1978,2670-2680). */
static void texel_rgba8(const swgb_texture *t, const swgb_texture_level *lv, uint16_t u, uint16_t v, uint16_t out[4])
{
    uint16_t xi = mulhi_u16(u, (uint16_t)lv->width);
    uint16_t yi = mulhi_u16(v, (uint16_t)lv->height);
    int32_t index = (int32_t)(int16_t)xi * 1 + (int32_t)(int16_t)yi * (int32_t)(int16_t)lv->pitch_texels; /* pmaddwd */
    const uint8_t *p = (const uint8_t *)lv->buffer + (size_t)(uint32_t)index * 4;
    const int bgra = t->format == SWGB_FORMAT_B8G8R8A8_UNORM || t->format == SWGB_FORMAT_B8G8R8A8_SRGB;
    const int srgb = t->format == SWGB_FORMAT_R8G8B8A8_SRGB || t->format == SWGB_FORMAT_B8G8R8A8_SRGB;
    for(int c = 0; c < 4; c++)
    {
        const uint8_t b = p[bgra ? bgra_byte(c) : c];
        out[c] = (srgb && c < 3) ? srgb_lut[b] : (uint16_t)(b << 8);
    }
}

/* sampleQuad2D for one lane (SamplerCore.cpp:668-909) */
static void sample_quad_2d(const OSampler *s, float u, float v, float lod, int secondLOD, uint16_t out[4], uint32_t *lvMask)
{
    int ilod = s->mipLinear ? trunc_int(lod) : round_int(lod); /* selectMipmap (:2357-2379) */
    const swgb_texture_level *lv = level_at(s, ilod + secondLOD);
    if(lvMask) *lvMask |= 1u << (uint32_t)(lv - s->t->levels);
    uint16_t uuuu = address16(u, s->t->address_u);
    uint16_t vvvv = address16(v, s->t->address_v);
    if(!s->linearFilter)
    {
        texel_rgba8(s->t, lv, uuuu, vvvv, out);
        return;
    }
    /* WriteTextureLevelInfo: uHalf = 0x8000 / width (VkDescriptorSetLayout.cpp:316-321) */
    uint16_t uHalf = (uint16_t)(0x8000 / lv->width);
    uint16_t vHalf = (uint16_t)(0x8000 / lv->height);
    int wrapU = s->t->address_u == SWGB_ADDRESS_REPEAT;
    int wrapV = s->t->address_v == SWGB_ADDRESS_REPEAT;
    uint16_t u0 = offset_sample(uuuu, uHalf, wrapU, -1);
    uint16_t v0 = offset_sample(vvvv, vHalf, wrapV, -1);
    uint16_t u1 = offset_sample(uuuu, uHalf, wrapU, +1);
    uint16_t v1 = offset_sample(vvvv, vHalf, wrapV, +1);
    uint16_t c00[4], c10[4], c01[4], c11[4];
    texel_rgba8(s->t, lv, u0, v0, c00);
    texel_rgba8(s->t, lv, u1, v0, c10);
    texel_rgba8(s->t, lv, u0, v1, c01);
    texel_rgba8(s->t, lv, u1, v1, c11);
    /* bilinearInterpolate, 8-bit unsigned components (:516-575) */
    uint16_t f0u = (uint16_t)(u0 * (uint16_t)lv->width);
    uint16_t f0v = (uint16_t)(v0 * (uint16_t)lv->height);
    uint16_t f1u = (uint16_t)~f0u, f1v = (uint16_t)~f0v;
    uint16_t f0u0v = mulhi_u16(f0u, f0v);
    uint16_t f1u0v = mulhi_u16(f1u, f0v);
    uint16_t f0u1v = mulhi_u16(f0u, f1v);
    uint16_t f1u1v = mulhi_u16(f1u, f1v);
    for(int c = 0; c < 4; c++)
    {
        uint16_t a = mulhi_u16(c00[c], f1u1v);
        uint16_t b = mulhi_u16(c10[c], f0u1v);
        uint16_t e = mulhi_u16(c01[c], f1u0v);
        uint16_t g = mulhi_u16(c11[c], f0u0v);
        out[c] = (uint16_t)((uint16_t)(a + b) + (uint16_t)(e + g));
    }
}

/* computeLod2D, implicit (SamplerCore.cpp:1376-1422) */
static float lod_2d(const OSampler *s, const float u[4], const float v[4])
{
    float dudx = fsub(u[1], u[0]), dudy = fsub(u[2], u[0]);
    float dvdx = fsub(v[1], v[0]), dvdy = fsub(v[2], v[0]);
    float a = fmul(dudx, s->W), b = fmul(dudy, s->W);
    float c = fmul(dvdx, s->H), e = fmul(dvdy, s->H);
    a = fmul(a, a); b = fmul(b, b); c = fmul(c, c); e = fmul(e, e);
    float lx = fadd(a, c), ly = fadd(b, e);
    float lod = fmaxr(lx, ly);
    return log2sqrt(lod);
}

/* halfToFloatBits (src/Pipeline/ShaderCore.cpp:627-645): texel conversion of
 * R16G16B16A16_SFLOAT textures. */
static float half_bits_to_float(uint16_t h)
{
    uint32_t sign16 = h & 0x8000u, man16 = h & 0x03FFu, exp16 = h & 0x7C00u;
    uint32_t sign32 = sign16 << 16, man32 = man16 << 13, exp32 = (exp16 + 0x1C000u) << 13;
    uint32_t norm32 = (man32 | exp32) | (exp16 == 0x7C00u ? 0x7F800000u : 0u);
    uint32_t magic = 126u << 23;
    uint32_t denorm32 = f2u(fsub(u2f(magic + man16), u2f(magic)));
    return u2f(sign32 | (exp16 == 0 ? denorm32 : norm32));
}

/* Float4 Frac (LLVMReactor.cpp:3252-3275): x - floor(x), at most 0x3F7FFFFF. */
static float frac4(float x)
{
    x = daz(x);
    return fminr(fsub(x, floorf(x)), u2f(0x3F7FFFFF));
}

/* address() for normalized float coordinates (SamplerCore.cpp:2463-2638). */
static void address_float(const OSampler *s, float coord, uint32_t mode, int dim, int32_t *x0, int32_t *x1, float *f)
{
    const float one = u2f(0x3F7FFFFF);
    if(mode == SWGB_ADDRESS_CLAMP_TO_EDGE)
        coord = fminr(fmaxr(coord, 0.0f), one);
    else if(mode == SWGB_ADDRESS_MIRRORED_REPEAT)
    {
        coord = fmul(coord, 0.5f);
        coord = fmul(2.0f, fabsf(fsub(coord, rintf(daz(coord)))));
        coord = fminr(coord, one);
    }
    else if(mode == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE)
        coord = fminr(fabsf(daz(coord)), one);
    else if(mode != SWGB_ADDRESS_CLAMP_TO_BORDER) /* ADDRESSING_BORDER: unmapped */
        coord = frac4(coord);
    coord = fmul(coord, (float)dim);
    if(mode == SWGB_ADDRESS_CLAMP_TO_BORDER)
    {
        /* point: Int4(Floor(coord)); linear: floor of coord - 0.5; then any
         * coordinate outside [0, dim) becomes -1 (SamplerCore.cpp:2568-2612) */
        if(!s->linearFilter)
        {
            *x0 = trunc_int(floorf(daz(coord)));
            *f = 0.0f;
        }
        else
        {
            coord = fsub(coord, 0.5f);
            float fl = floorf(daz(coord));
            *x0 = trunc_int(fl);
            *f = fsub(coord, fl);
        }
        *x1 = *x0 + 1;
        if(*x0 < 0 || *x0 >= dim) *x0 = -1;
        if(*x1 < 0 || *x1 >= dim) *x1 = -1;
        return;
    }
    if(!s->linearFilter)
    {
        *x0 = trunc_int(coord);
        *x1 = *x0 + 1;
        *f = 0.0f;
        return;
    }
    coord = fsub(coord, 0.5f);
    float fl = floorf(daz(coord));
    *x0 = trunc_int(fl);
    *f = fsub(coord, fl);
    *x1 = *x0 + 1;
    if(mode == SWGB_ADDRESS_REPEAT)
    {
        if(*x0 < 0) *x0 = dim - 1;
        if(!(*x1 < dim)) *x1 = 0;
    }
    else
    {
        if(*x0 < 0) *x0 = 0;
        if(*x1 > dim - 1) *x1 = dim - 1;
    }
}

static void texel_float(const swgb_texture *t, const swgb_texture_level *lv, int32_t index, float out[4])
{
    if(is_tex8(t->format))
    {
        /* an 8-bit texture on the 32-bit path (border addressing): the 16-bit
         * sampleTexel's components as floats (SamplerCore.cpp:2215-2245) */
        const uint8_t *p = (const uint8_t *)lv->buffer + (size_t)(uint32_t)index * 4;
        const int bgra = t->format == SWGB_FORMAT_B8G8R8A8_UNORM || t->format == SWGB_FORMAT_B8G8R8A8_SRGB;
        const int srgb = t->format == SWGB_FORMAT_R8G8B8A8_SRGB || t->format == SWGB_FORMAT_B8G8R8A8_SRGB;
        for(int c = 0; c < 4; c++)
        {
            const uint8_t b = p[bgra ? bgra_byte(c) : c];
            out[c] = (float)((srgb && c < 3) ? srgb_lut[b] : (uint16_t)(b << 8));
        }
        return;
    }
    if(t->format == SWGB_FORMAT_R32G32B32A32_SFLOAT)
        memcpy(out, (const uint8_t *)lv->buffer + (size_t)(uint32_t)index * 16, 16);
    else
    {
        const uint16_t *p = (const uint16_t *)((const uint8_t *)lv->buffer + (size_t)(uint32_t)index * 8);
        for(int c = 0; c < 4; c++) out[c] = half_bits_to_float(p[c]);
    }
}

/* sampleTexel of the 32-bit path (SamplerCore.cpp:2093-2110,1645-1677,
 * 2290-2355): with border addressing, a texel whose coordinate is -1 (u, or
 * v times the pitch, negative) is read at index 0 and replaced by the border
 * colour, given in the path's units (scaled by getComponentScale()). */
static void border_texel(const OSampler *s, const swgb_texture_level *lv, int32_t x, int32_t ypitch, float out[4])
{
    const int border = s->t->address_u == SWGB_ADDRESS_CLAMP_TO_BORDER || s->t->address_v == SWGB_ADDRESS_CLAMP_TO_BORDER;
    const int valid = !border || (x | ypitch) >= 0;
    texel_float(s->t, lv, valid ? x + ypitch : 0, out);
    if(valid) return;
    const float sc = is_tex8(s->t->format) ? 65280.0f : 1.0f;
    switch(s->t->border_color)
    {
    case SWGB_BORDER_COLOR_FLOAT_OPAQUE_BLACK: out[0] = out[1] = out[2] = 0.0f; out[3] = sc; break;
    case SWGB_BORDER_COLOR_FLOAT_OPAQUE_WHITE: out[0] = out[1] = out[2] = out[3] = sc; break;
    case SWGB_BORDER_COLOR_FLOAT_CUSTOM_EXT:
        for(int c = 0; c < 4; c++) out[c] = sc * s->t->custom_border_color[c];
        break;
    default: out[0] = out[1] = out[2] = out[3] = 0.0f; break;
    }
}

/* sampleFloat2D for one lane (SamplerCore.cpp:1155-1248). */
static void sample_float_2d(const OSampler *s, float u, float v, float lod, int secondLOD, float out[4], uint32_t *lvMask)
{
    int ilod = s->mipLinear ? trunc_int(lod) : round_int(lod);
    const swgb_texture_level *lv = level_at(s, ilod + secondLOD);
    if(lvMask) *lvMask |= 1u << (uint32_t)(lv - s->t->levels);
    int32_t x0, x1, y0, y1;
    float fu, fv;
    address_float(s, u, s->t->address_u, (int)lv->width, &x0, &x1, &fu);
    address_float(s, v, s->t->address_v, (int)lv->height, &y0, &y1, &fv);
    int32_t pitch = (int32_t)lv->pitch_texels;
    y0 *= pitch;
    y1 *= pitch;
    float c00[4], c10[4], c01[4], c11[4];
    if(!s->linearFilter)
    {
        border_texel(s, lv, x0, y0, out);
        return;
    }
    border_texel(s, lv, x0, y0, c00);
    border_texel(s, lv, x1, y0, c10);
    border_texel(s, lv, x0, y1, c01);
    border_texel(s, lv, x1, y1, c11);
    for(int c = 0; c < 4; c++)
    {
        float a = fadd(c00[c], fmul(fu, fsub(c10[c], c00[c])));
        float b = fadd(c01[c], fmul(fu, fsub(c11[c], c01[c])));
        out[c] = fadd(a, fmul(fv, fsub(b, a)));
    }
}

/* sampleTexture128 for the 16-bit path (SamplerCore.cpp:59-253): returns
 * 4 lanes x RGBA, scaled by 1/getComponentScale() = 1/0xFF00. */
static void sample_texture_quad(const OSampler *s, const float u[4], const float v[4], float out[4][4], uint32_t *lvMask)
{
    float lod;
    if(s->minLod == s->maxLod)
        lod = s->minLod;
    else
    {
        lod = lod_2d(s, u, v);
        lod = fadd(lod, s->bias);
        lod = fmaxr(lod, s->minLod);
        lod = fminr(lod, s->maxLod);
    }
    const int border = s->t->address_u == SWGB_ADDRESS_CLAMP_TO_BORDER || s->t->address_v == SWGB_ADDRESS_CLAMP_TO_BORDER;
    if(!is_tex8(s->t->format) || border)
    {
        /* sampleFloatFilter (SamplerCore.cpp:1061-1083); border addressing
         * selects this 32-bit path for every format (:173-176), and 8-bit
         * texels are normalized by 1 / 0xFF00 after it (:200-209) */
        float fr = fsub(daz(lod), floorf(daz(lod))); /* scalar Frac: lod - floor(lod) */
        for(int lane = 0; lane < 4; lane++)
        {
            float c[4];
            sample_float_2d(s, u[lane], v[lane], lod, 0, c, lvMask);
            if(s->mipLinear)
            {
                float cc[4];
                sample_float_2d(s, u[lane], v[lane], lod, 1, cc, lvMask);
                for(int k = 0; k < 4; k++) c[k] = fadd(fmul(fsub(cc[k], c[k]), fr), c[k]);
            }
            for(int k = 0; k < 4; k++) out[lane][k] = is_tex8(s->t->format) ? fmul(c[k], 1.0f / 65280.0f) : c[k];
        }
        return;
    }
    const float scale = 1.0f / 65280.0f;
    for(int lane = 0; lane < 4; lane++)
    {
        uint16_t c[4];
        sample_quad_2d(s, u[lane], v[lane], lod, 0, c, lvMask);
        if(s->mipLinear) /* sampleFilter trilinear (:324-379) */
        {
            uint16_t cc[4];
            sample_quad_2d(s, u[lane], v[lane], lod, 1, cc, lvMask);
            float l = fmul(lod, 65536.0f);
            uint16_t utri = (uint16_t)trunc_int(l);
            for(int k = 0; k < 4; k++) cc[k] = mulhi_u16(cc[k], utri);
            utri = (uint16_t)~utri;
            for(int k = 0; k < 4; k++) c[k] = (uint16_t)(mulhi_u16(c[k], utri) + cc[k]);
        }
        for(int k = 0; k < 4; k++) out[lane][k] = fmul((float)c[k], scale);
    }
}

swgb_status oracle_sample_quad(const swgb_texture *tex, const float u[4], const float v[4], float out[16])
{
    pthread_once(&srgb_once, srgb_init); /* sRGB textures decode through the table prepare() builds for draws */
    OSampler s;
    sampler_init(&s, tex);
    float o[4][4];
    sample_texture_quad(&s, u, v, o, NULL);
    for(int l = 0; l < 4; l++)
        for(int c = 0; c < 4; c++) out[l * 4 + c] = o[l][c];
    return SWGB_OK;
}

/* ------------------------------------------------------------------------ */
/* Pixel stage (QuadRasterizer.cpp:71-250, PixelRoutine.cpp:97-358,         */
/* PixelProgram.cpp:138-364, PixelRoutine.cpp:494-739,1225-2700)             */
/* ------------------------------------------------------------------------ */

static float blend_factor(uint32_t f, const float src[4], const float dst[4], int comp)
{
    /* blendFactorRGB / blendFactorAlpha (PixelRoutine.cpp:1225-1393); the
     * [0,1] clamp of ONE_MINUS_* applies to SNORM only, none here. */
    int alpha = comp == 3;
    switch(f)
    {
    case SWGB_BLEND_ZERO: return 0.0f;
    case SWGB_BLEND_ONE: return 1.0f;
    case SWGB_BLEND_SRC_COLOR: return alpha ? src[3] : src[comp];
    case SWGB_BLEND_ONE_MINUS_SRC_COLOR: return fsub(1.0f, alpha ? src[3] : src[comp]);
    case SWGB_BLEND_DST_COLOR: return alpha ? dst[3] : dst[comp];
    case SWGB_BLEND_ONE_MINUS_DST_COLOR: return fsub(1.0f, alpha ? dst[3] : dst[comp]);
    case SWGB_BLEND_SRC_ALPHA: return src[3];
    case SWGB_BLEND_ONE_MINUS_SRC_ALPHA: return fsub(1.0f, src[3]);
    case SWGB_BLEND_DST_ALPHA: return dst[3];
    case SWGB_BLEND_ONE_MINUS_DST_ALPHA: return fsub(1.0f, dst[3]);
    default: return 0.0f;
    }
}

static float blend_op(uint32_t op, float s, float sf, float dd, float df)
{
    switch(op)
    {
    case SWGB_BLEND_OP_ADD: return fadd(fmul(s, sf), fmul(dd, df));
    case SWGB_BLEND_OP_SUBTRACT: return fsub(fmul(s, sf), fmul(dd, df));
    case SWGB_BLEND_OP_REVERSE_SUBTRACT: return fsub(fmul(dd, df), fmul(s, sf));
    case SWGB_BLEND_OP_MIN: return fminr(s, dd);
    case SWGB_BLEND_OP_MAX: return fmaxr(s, dd);
    case OP_SRC_EXT: return s;
    case OP_DST_EXT: return dd;
    case OP_ZERO_EXT: return 0.0f;
    default: return s;
    }
}

/* R16G16B16A16_SFLOAT attachments: the blend reads with Reactor's
 * Float(Half) (src/Reactor/Reactor.cpp:3787-3815; a half infinity/NaN reads as
 * 65536 + ...), and writeColor stores Half(Float) (:3744-3770). */
static float half_to_float(uint16_t h)
{
    int32_t fp16i = h;
    int32_t sgn = (fp16i >> 15) & 1, e = (fp16i >> 10) & 0x1F, m = fp16i & 0x3FF;
    uint32_t fp32i = (uint32_t)sgn << 31;
    if(e == 0)
    {
        if(m != 0)
        {
            while((m & 0x400) == 0)
            {
                m <<= 1;
                e -= 1;
            }
            fp32i |= (uint32_t)(((e + (127 - 15) + 1) << 23) | ((m & ~0x400) << 13));
        }
    }
    else
        fp32i |= (uint32_t)(((e + (127 - 15)) << 23) | (m << 13));
    return u2f(fp32i);
}

static uint16_t float_to_half(float f)
{
    uint32_t fp32i = f2u(f);
    uint32_t ab = fp32i & 0x7FFFFFFFu;
    uint16_t fp16i = (uint16_t)((fp32i & 0x80000000u) >> 16);
    if(ab > 0x47FFEFFFu)
        fp16i |= 0x7FFF;
    else if(ab < 0x38800000u)
    {
        int32_t mantissa = (int32_t)((ab & 0x007FFFFFu) | 0x00800000u);
        int32_t e = 113 - (int32_t)(ab >> 23);
        uint32_t a2 = e < 24 ? (uint32_t)(mantissa >> e) : 0u;
        fp16i |= (uint16_t)((a2 + 0x00000FFFu + ((a2 >> 13) & 1u)) >> 13);
    }
    else
        fp16i |= (uint16_t)((ab + 0xC8000000u + 0x00000FFFu + ((ab >> 13) & 1u)) >> 13);
    return fp16i;
}

static void read_color(const ODraw *d, int q, int x, int y, float dst[4])
{
    const swgb_pipeline_state *st = d->st;
    uint8_t *row = (uint8_t *)st->color + (size_t)q * st->color_slice_bytes + (size_t)y * st->color_pitch_bytes;
    if(is_unorm(st->color_format))
    {
        /* readPixel (PixelRoutine.cpp:1091-1130) widens b to b*257; alphaBlend
         * scales by 1/0xFFFF and decodes sRGB R, G, B (:1812-1828); B8G8R8A8
         * swaps R and B. */
        const uint8_t *p = row + (size_t)x * 4;
        const int bgra = is_bgra(st->color_format);
        for(int c = 0; c < 4; c++) dst[c] = fmul((float)(p[bgra ? bgra_byte(c) : c] * 257), 1.0f / 0xFFFF);
        if(is_srgb(st->color_format))
            for(int c = 0; c < 3; c++) dst[c] = srgb_to_linear(dst[c]);
    }
    else if(st->color_format == SWGB_FORMAT_R32G32B32A32_SFLOAT)
        memcpy(dst, row + (size_t)x * 16, 16);
    else
    {
        const uint16_t *p = (const uint16_t *)(row + (size_t)x * 8);
        for(int c = 0; c < 4; c++) dst[c] = half_to_float(p[c]);
    }
}

static void write_color(const ODraw *d, int q, int x, int y, const float col[4])
{
    const swgb_pipeline_state *st = d->st;
    uint8_t *row = (uint8_t *)st->color + (size_t)q * st->color_slice_bytes + (size_t)y * st->color_pitch_bytes;
    uint32_t wm = st->color_write_mask;
    if(is_unorm(st->color_format))
    {
        /* writeColor (PixelRoutine.cpp:1963-1993,2603-2650): sRGB encodes R, G,
         * B first; B8G8R8A8 swaps R and B, and their write-mask bits with
         * them (:2138-2143) */
        uint8_t *p = row + (size_t)x * 4;
        const int bgra = is_bgra(st->color_format), srgb = is_srgb(st->color_format);
        for(int c = 0; c < 4; c++)
        {
            float v = fminr(fmaxr((srgb && c < 3) ? linear_to_srgb(col[c]) : col[c], 0.0f), 1.0f);
            int32_t r = round_int(fmul(v, 255.0f));
            int16_t s16 = (int16_t)r;
            uint8_t b = s16 < 0 ? 0 : (s16 > 255 ? 255 : (uint8_t)s16); /* PackUnsigned */
            if(wm & (1u << c)) p[bgra ? bgra_byte(c) : c] = b;
        }
    }
    else if(st->color_format == SWGB_FORMAT_R32G32B32A32_SFLOAT)
    {
        float *p = (float *)(row + (size_t)x * 16);
        for(int c = 0; c < 4; c++)
            if(wm & (1u << c)) p[c] = col[c];
    }
    else
    {
        uint16_t *p = (uint16_t *)(row + (size_t)x * 8);
        for(int c = 0; c < 4; c++)
            if(wm & (1u << c)) p[c] = float_to_half(col[c]);
    }
}

static void *depth_at(const ODraw *d, int q, int x, int y)
{
    const swgb_pipeline_state *st = d->st;
    return (uint8_t *)st->depth + (size_t)q * st->depth_slice_bytes + (size_t)y * st->depth_pitch_bytes + (size_t)x * (d16(st) ? 2 : 4);
}

/* Stored depth as the test compares it: D32_SFLOAT as is, D16_UNORM as the
 * float of its integer (readDepth16, PixelRoutine.cpp:465-481). */
static float read_depth(const ODraw *d, int q, int x, int y)
{
    if(d16(d->st)) return (float)*(const uint16_t *)depth_at(d, q, x, y);
    return *(const float *)depth_at(d, q, x, y);
}

/* The fragment depth the test uses: Z for D32_SFLOAT, for D16_UNORM
 * Min(Max(Round(Z * 0xFFFF), 0), 0xFFFF) (PixelRoutine.cpp:506-510); writeDepth16
 * stores the same integer (:687-713). */
static float depth_value(const ODraw *d, float Z)
{
    if(!d16(d->st)) return Z;
    return fminr(fmaxr(nearbyintf(fmul(Z, 65535.0f)), 0.0f), 65535.0f);
}

/* depthBoundsTest16 / 32F (PixelRoutine.cpp:576-609): the stored value, D16
 * scaled by 1/0xFFFF, within [minDepthBounds, maxDepthBounds]. */
static int bounds_pass(const ODraw *d, float stored)
{
    const float z = d16(d->st) ? fmul(stored, 1.0f / 0xFFFF) : stored;
    return fle(d->st->min_depth_bounds, z) && fle(z, d->st->max_depth_bounds);
}

static uint8_t *stencil_at(const ODraw *d, int q, int x, int y)
{
    const swgb_pipeline_state *st = d->st;
    return (uint8_t *)st->stencil + (size_t)q * st->stencil_slice_bytes + (size_t)y * st->stencil_pitch_bytes + (size_t)x;
}

/* stencilTest (:360-449): (reference & compareMask) op (stored & compareMask) */
static int stencil_pass(const swgb_stencil_op_state *s, uint32_t stored)
{
    const uint32_t m = s->compare_mask & 0xFFu, r = s->reference & m, v = stored & m;
    switch(s->compare_op)
    {
    case SWGB_COMPARE_NEVER: return 0;
    case SWGB_COMPARE_LESS: return r < v;
    case SWGB_COMPARE_EQUAL: return r == v;
    case SWGB_COMPARE_LESS_OR_EQUAL: return r <= v;
    case SWGB_COMPARE_GREATER: return r > v;
    case SWGB_COMPARE_NOT_EQUAL: return r != v;
    case SWGB_COMPARE_GREATER_OR_EQUAL: return r >= v;
    default: return 1;
    }
}

/* stencilOperation (:862-895), 8-bit with saturation / wrap */
static uint32_t stencil_op(const swgb_stencil_op_state *s, uint32_t op, uint32_t v)
{
    switch(op)
    {
    case SWGB_STENCIL_OP_ZERO: return 0;
    case SWGB_STENCIL_OP_REPLACE: return s->reference & 0xFFu;
    case SWGB_STENCIL_OP_INCREMENT_AND_CLAMP: return v < 255 ? v + 1 : 255;
    case SWGB_STENCIL_OP_DECREMENT_AND_CLAMP: return v > 0 ? v - 1 : 0;
    case SWGB_STENCIL_OP_INVERT: return (~v) & 0xFFu;
    case SWGB_STENCIL_OP_INCREMENT_AND_WRAP: return (v + 1) & 0xFFu;
    case SWGB_STENCIL_OP_DECREMENT_AND_WRAP: return (v - 1) & 0xFFu;
    default: return v;
    }
}

static void write_depth(const ODraw *d, int q, int x, int y, float Z)
{
    if(d16(d->st)) *(uint16_t *)depth_at(d, q, x, y) = (uint16_t)Z;
    else *(float *)depth_at(d, q, x, y) = Z;
}

/* One 2x2 quad of one primitive (PixelRoutine::quad :97-358); cMask[q] holds
 * the lane coverage of sample q.  The shader runs once per quad at the pixel
 * centres (no per-sample shading); depth and colour are per sample. */
static void pixel_quad(const ODraw *d, const OSampler *smp, const OPrim *pr, int x, int y, const int cMask[4], swgb_counters *cnt)
{
    const swgb_pipeline_state *st = d->st;
    float xF[4], yF[4];
    for(int i = 0; i < 4; i++)
    {
        xF[i] = fsub(fadd((float)x, (float)(i & 1)), pr->x0);
        yF[i] = fsub(fadd((float)y, (float)(i >> 1)), pr->y0);
    }
    float z[4][4] = { { 0 } };
    if(d->interpolateZ)
        for(int q = 0; q < d->ms; q++)
            for(int i = 0; i < 4; i++)
            {
                float yq = yF[i], xq = xF[i];
                if(d->ms > 1)
                {
                    yq = fadd(yq, SLY[q]); /* QuadRasterizer.cpp:131-141 */
                    xq = fsub(xq, SLX[q]); /* PixelRoutine.cpp:128-148 */
                }
                float Dz = fadd(pr->z.C, fmul(yq, pr->z.B));
                z[q][i] = interp_muladd(xq, pr->z.A, Dz);
                if(d->st->depth_bias_constant != 0.0f || d->st->depth_bias_slope != 0.0f)
                    z[q][i] = fadd(z[q][i], pr->zBias); /* PixelRoutine.cpp:141-144 */
            }
    /* w, rhw (:196-199) and varyings (:231-261) */
    float rhw[4];
    for(int i = 0; i < 4; i++)
    {
        float Dw = fadd(pr->w.C, fmul(yF[i], pr->w.B));
        float w = interp_muladd(xF[i], pr->w.A, Dw);
        rhw[i] = fdiv(1.0f, w);
    }
    float vin[MAXV][4];
    for(int k = 0; k < d->nv; k++)
        for(int i = 0; i < 4; i++)
        {
            float Dv = fadd(pr->V[k].C, fmul(yF[i], pr->V[k].B));
            vin[k][i] = fmul(interp_muladd(xF[i], pr->V[k].A, Dv), rhw[i]);
        }
    /* Fixed fragment shader (PixelProgram::executeShader :138-241) */
    float c[4][4];
    if(st->fragment_shader == SWGB_FS_TEX_X_VCOLOR)
    {
        float tex[4][4];
        uint32_t m = 0;
        sample_texture_quad(smp, vin[4], vin[5], tex, &m);
        if(cnt) cnt->texture_levels_mask |= m;
        for(int i = 0; i < 4; i++)
            for(int k = 0; k < 4; k++) c[i][k] = fmul(tex[i][k], vin[k][i]);
    }
    else
        for(int i = 0; i < 4; i++)
            for(int k = 0; k < 4; k++) c[i][k] = vin[k][i];
    /* clampColor (PixelProgram.cpp:286-364) */
    if(is_unorm(st->color_format))
        for(int i = 0; i < 4; i++)
            for(int k = 0; k < 4; k++) c[i][k] = fminr(fmaxr(c[i][k], 0.0f), 1.0f);

    for(int q = 0; q < d->ms; q++)
    {
        /* stencilTest (:360-449): sMask */
        const int stencilOn = st->stencil && st->stencil_test_enable;
        const swgb_stencil_op_state *so = pr->front ? &st->front : &st->back;
        int sMask = cMask[q];
        uint8_t sv[4] = { 0, 0, 0, 0 };
        if(stencilOn)
            for(int i = 0; i < 4; i++)
            {
                if(!(cMask[q] & (1 << i))) continue;
                sv[i] = *stencil_at(d, q, x + (i & 1), y + (i >> 1));
                if(!stencil_pass(so, sv[i])) sMask &= ~(1 << i);
            }
        int covered = cMask[q];
        /* late depth test (:330-344), depth write (:715-739) */
        int zMask = cMask[q];
        if(d->depthTest)
        {
            zMask = 0;
            for(int i = 0; i < 4; i++)
            {
                if(!(cMask[q] & (1 << i))) continue;
                float Z = z[q][i];
                if(d->depthClamp) Z = fminr(fmaxr(Z, d->minDepthClamp), d->maxDepthClamp);
                Z = depth_value(d, Z);
                z[q][i] = Z;
                float zb = read_depth(d, q, x + (i & 1), y + (i >> 1));
                int pass;
                switch(st->depth_compare_op)
                {
                case SWGB_COMPARE_NEVER: pass = 0; break;
                case SWGB_COMPARE_LESS: pass = !fle(zb, Z); break;
                case SWGB_COMPARE_EQUAL: pass = feq(zb, Z); break;
                case SWGB_COMPARE_LESS_OR_EQUAL: pass = !flt(zb, Z); break;
                case SWGB_COMPARE_GREATER: pass = flt(zb, Z); break;
                case SWGB_COMPARE_NOT_EQUAL: pass = !feq(zb, Z); break;
                case SWGB_COMPARE_GREATER_OR_EQUAL: pass = fle(zb, Z); break;
                default: pass = 1; break;
                }
                /* depthBoundsTest after the depth test, on the stored value (:576-640) */
                if(pass && st->depth_bounds_test_enable && !bounds_pass(d, zb)) pass = 0;
                if(pass) zMask |= 1 << i;
            }
            if(stencilOn) zMask &= sMask; /* depthTest ends with zMask &= sMask (:571-574) */
            if(cnt) cnt->fragments_tested += (uint64_t)__builtin_popcount((unsigned)cMask[q]);
            if(d->depthWrite)
                for(int i = 0; i < 4; i++)
                    if(zMask & (1 << i)) write_depth(d, q, x + (i & 1), y + (i >> 1), z[q][i]);
        }
        else if(st->depth_bounds_test_enable && st->depth)
        {
            /* no depth test: the bounds test masks the coverage (:626-629) */
            for(int i = 0; i < 4; i++)
                if((covered & (1 << i)) && !bounds_pass(d, read_depth(d, q, x + (i & 1), y + (i >> 1)))) covered &= ~(1 << i);
            zMask = covered;
        }
        if(stencilOn)
        {
            /* writeStencil (:754-860): failOp where the stencil test failed,
             * depthFailOp where the depth test did, passOp else; write mask */
            for(int i = 0; i < 4; i++)
            {
                if(!(covered & (1 << i))) continue;
                uint32_t op = !(sMask & (1 << i)) ? so->fail_op : ((d->depthTest && !(zMask & (1 << i))) ? so->depth_fail_op : so->pass_op);
                uint32_t wm = so->write_mask & 0xFFu;
                uint32_t nv = stencil_op(so, op, sv[i]);
                *stencil_at(d, q, x + (i & 1), y + (i >> 1)) = (uint8_t)((nv & wm) | (sv[i] & ~wm));
            }
            zMask &= sMask; /* writeColor: xMask &= sMask (:2156-2159) */
        }
        if(cnt) cnt->fragments_passed += (uint64_t)__builtin_popcount((unsigned)zMask);
        if(d->vis)
            for(int i = 0; i < 4; i++)
            {
                if(!(zMask & (1 << i))) continue;
                size_t pix = ((size_t)q * st->framebuffer_height + (size_t)(y + (i >> 1))) * st->framebuffer_width + (size_t)(x + (i & 1));
                uint32_t n = d->visLen[pix]++;
                if(n < (uint32_t)d->visCap) d->vis[pix * (size_t)d->visCap + n] = pr->id;
            }

        /* blendColor / alphaBlend / writeColor per sample plane (PixelProgram.cpp:261-284) */
        for(int i = 0; i < 4; i++)
        {
            if(!(zMask & (1 << i))) continue;
            int px = x + (i & 1), py = y + (i >> 1);
            float out[4];
            if(d->blend)
            {
                float dst[4];
                read_color(d, q, px, py, dst);
                float sf[4], df[4];
                for(int k = 0; k < 3; k++)
                {
                    sf[k] = blend_factor(d->srcC, c[i], dst, k);
                    df[k] = blend_factor(d->dstC, c[i], dst, k);
                }
                sf[3] = blend_factor(d->srcA, c[i], dst, 3);
                df[3] = blend_factor(d->dstA, c[i], dst, 3);
                for(int k = 0; k < 3; k++) out[k] = blend_op(d->opC, c[i][k], sf[k], dst[k], df[k]);
                out[3] = blend_op(d->opA, c[i][3], sf[3], dst[3], df[3]);
            }
            else
                memcpy(out, c[i], sizeof(out));
            write_color(d, q, px, py, out);
        }
    }
}

/* QuadRasterizer::generate/rasterize for one cluster (QuadRasterizer.cpp:36-233). */
static void raster_cluster(const ODraw *d, const OSampler *smp, const OPrim *pr, int cluster, int clusterCount, swgb_counters *cnt)
{
    if(!pr->visible) return;
    int yMin = pr->yMin, yMax = pr->yMax;
    int cluster2 = cluster + cluster;
    yMin += clusterCount * 2 - 2 - cluster2;
    yMin &= -clusterCount * 2;
    yMin += cluster2;
    for(int y = yMin; y < yMax; y += 2 * clusterCount)
    {
        int x0 = 0x7FFFFFFF, x1 = -0x7FFFFFFF;
        int16_t xl[4][4], xr[4][4];
        for(int q = 0; q < d->ms; q++)
        {
            int l0 = pr->left[q][y + 1], l1 = pr->left[q][y + 2];
            int r0 = pr->right[q][y + 1], r1 = pr->right[q][y + 2];
            int a = l0 < l1 ? l0 : l1, b = r0 > r1 ? r0 : r1;
            x0 = a < x0 ? a : x0;
            x1 = b > x1 ? b : x1;
            xl[q][0] = (int16_t)(l0 - 1); xl[q][1] = (int16_t)(l0 - 2); xl[q][2] = (int16_t)(l1 - 1); xl[q][3] = (int16_t)(l1 - 2);
            xr[q][0] = (int16_t)(r0 - 0); xr[q][1] = (int16_t)(r0 - 1); xr[q][2] = (int16_t)(r1 - 0); xr[q][3] = (int16_t)(r1 - 1);
        }
        x0 &= ~1;
        for(int x = x0; x < x1; x += 2)
        {
            int16_t xx = (int16_t)x;
            int cMask[4] = { 0, 0, 0, 0 }, any = 0;
            for(int q = 0; q < d->ms; q++)
            {
                for(int i = 0; i < 4; i++)
                    if(xx > xl[q][i] && xr[q][i] > xx) cMask[q] |= 1 << i;
                any |= cMask[q];
            }
            if(any == 0) continue;
            if(cnt) cnt->quads++;
            pixel_quad(d, smp, pr, x, y, cMask, cnt);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Draw driver (Renderer::draw + DrawCall::run, Renderer.cpp:183-598)         */
/* ------------------------------------------------------------------------ */

#define BATCH 128      /* MaxBatchSize (src/Device/Renderer.hpp:50) */
#define CLUSTERS 16    /* MaxClusterCount (src/Device/Renderer.hpp:52) */
#define GROUP_BATCHES 64

typedef struct {
    const ODraw *d;
    const OSampler *smp;
    OPrim *prims;      /* GROUP_BATCHES * BATCH */
    uint16_t *spans;   /* per prim: 2 * rows */
    uint32_t first, count;
    int phase;         /* 0 setup, 1 pixels */
    int nthreads;
    int next;          /* work counter (protected by mutex) */
    pthread_mutex_t mu;
    swgb_counters local[64];
    int clipped_count[64];
} OJob;

static void run_setup(OJob *j, int t)
{
    const ODraw *d = j->d;
    for(;;)
    {
        pthread_mutex_lock(&j->mu);
        int b = j->next++;
        pthread_mutex_unlock(&j->mu);
        uint32_t start = (uint32_t)b * BATCH;
        if(start >= j->count) break;
        uint32_t end = start + BATCH < j->count ? start + BATCH : j->count;
        for(uint32_t i = start; i < end; i++)
        {
            OPrim *pr = &j->prims[i];
            for(int q = 0; q < 4; q++)
            {
                pr->left[q] = j->spans + ((size_t)i * 8 + 2 * q) * d->rows;
                pr->right[q] = pr->left[q] + d->rows;
            }
            int clipped = 0;
            pr->id = j->first + i;
            int vis = process_triangle(d, j->first + i, pr, &j->local[t], &clipped);
            j->local[t].triangles_in++;
            if(clipped) j->local[t].triangles_clipped++;
            if(vis) j->local[t].triangles_visible++;
            else j->local[t].triangles_rejected++;
        }
    }
}

static void run_pixels(OJob *j, int t)
{
    for(;;)
    {
        pthread_mutex_lock(&j->mu);
        int c = j->next++;
        pthread_mutex_unlock(&j->mu);
        if(c >= CLUSTERS) break;
        for(uint32_t i = 0; i < j->count; i++) raster_cluster(j->d, j->smp, &j->prims[i], c, CLUSTERS, &j->local[t]);
    }
}

typedef struct { OJob *j; int t; } OArg;

static void *worker(void *p)
{
    OArg *a = (OArg *)p;
    if(a->j->phase == 0) run_setup(a->j, a->t);
    else run_pixels(a->j, a->t);
    return NULL;
}

static void run_phase(OJob *j, int phase)
{
    j->phase = phase;
    j->next = 0;
    int n = j->nthreads;
    if(n <= 1)
    {
        OArg a = { j, 0 };
        worker(&a);
        return;
    }
    pthread_t th[64];
    OArg args[64];
    for(int t = 0; t < n; t++)
    {
        args[t].j = j;
        args[t].t = t;
        pthread_create(&th[t], NULL, worker, &args[t]);
    }
    for(int t = 0; t < n; t++) pthread_join(th[t], NULL);
}

static swgb_status draw_impl(const swgb_pipeline_state *st, const swgb_draw_args *a, int nthreads, swgb_counters *cnt,
                             uint32_t *vis, uint32_t *visLen, int visCap);

/* ComputePrimitiveCount for the triangle topologies (src/Device/Context.cpp:26-46). */
static uint32_t primitive_count(uint32_t topology, uint32_t vertexCount)
{
    if(topology == SWGB_TOPOLOGY_TRIANGLE_LIST) return vertexCount / 3;
    return (vertexCount > 2 ? vertexCount : 2) - 2;
}

/* Primitive restart: vk::IndexBuffer::getIndexBuffers with
 * ProcessPrimitiveRestart (src/Device/Context.cpp:49-91,249-289) splits the
 * index stream at every all-ones index into sub-draws (primitive count, first
 * index); each is drawn in turn, as its own Renderer::draw. */
static swgb_status draw_restart(const swgb_pipeline_state *st, const swgb_draw_args *a, int nthreads, swgb_counters *cnt)
{
    const uint32_t bytes = a->index_type == SWGB_INDEX_TYPE_UINT8 ? 1u : (a->index_type == SWGB_INDEX_TYPE_UINT16 ? 2u : 4u);
    const uint32_t restart = bytes == 1 ? 0xFFu : (bytes == 2 ? 0xFFFFu : 0xFFFFFFFFu);
    uint32_t start = 0, vertexCount = 0;
    for(uint32_t i = 0; i <= a->restart_index_count; i++)
    {
        uint32_t v = restart;
        if(i < a->restart_index_count)
            v = bytes == 1 ? ((const uint8_t *)a->indices)[i] : (bytes == 2 ? ((const uint16_t *)a->indices)[i] : ((const uint32_t *)a->indices)[i]);
        if(v == restart)
        {
            const uint32_t prims = vertexCount ? primitive_count(st->topology, vertexCount) : 0;
            if(prims > 0)
            {
                swgb_draw_args sub = *a;
                sub.restart_index_count = 0;
                sub.count = prims;
                sub.indices = (const uint8_t *)a->indices + (size_t)start * bytes;
                swgb_status s = draw_impl(st, &sub, nthreads, cnt, NULL, NULL, 0);
                if(s != SWGB_OK) return s;
            }
            vertexCount = 0;
        }
        else
        {
            if(vertexCount == 0) start = i;
            vertexCount++;
        }
    }
    return SWGB_OK;
}

static swgb_status draw_impl(const swgb_pipeline_state *st, const swgb_draw_args *a, int nthreads, swgb_counters *cnt,
                             uint32_t *vis, uint32_t *visLen, int visCap)
{
    if(!st || !a) return SWGB_INVALID_ARG;
    if(a->restart_index_count && a->index_type != SWGB_INDEX_TYPE_NONE)
        return visCap > 0 ? SWGB_UNSUPPORTED_STATE : draw_restart(st, a, nthreads, cnt);
    if(a->count == 0) return SWGB_OK; /* Renderer.cpp:187 */
    ODraw d;
    swgb_status s = prepare(&d, st, a);
    if(s != SWGB_OK) return s;
    d.vis = visCap > 0 ? vis : NULL;
    d.visLen = visLen;
    d.visCap = visCap;
    if(!st->color) return SWGB_INVALID_ARG;
    OSampler smp;
    memset(&smp, 0, sizeof(smp));
    if(st->fragment_shader == SWGB_FS_TEX_X_VCOLOR) sampler_init(&smp, &st->texture);
    if(nthreads < 1) nthreads = 1;
    if(nthreads > 64) nthreads = 64;

    uint32_t group = GROUP_BATCHES * BATCH;
    OJob j;
    memset(&j, 0, sizeof(j));
    j.d = &d;
    j.smp = &smp;
    j.nthreads = nthreads;
    pthread_mutex_init(&j.mu, NULL);
    j.prims = (OPrim *)calloc(group, sizeof(OPrim));
    j.spans = (uint16_t *)malloc((size_t)group * 8 * d.rows * sizeof(uint16_t));
    if(!j.prims || !j.spans)
    {
        free(j.prims);
        free(j.spans);
        return SWGB_OOM;
    }
    for(uint32_t first = 0; first < a->count; first += group)
    {
        j.first = first;
        j.count = a->count - first < group ? a->count - first : group;
        run_phase(&j, 0);
        run_phase(&j, 1);
    }
    if(cnt)
        for(int t = 0; t < nthreads; t++)
        {
            cnt->triangles_in += j.local[t].triangles_in;
            cnt->triangles_rejected += j.local[t].triangles_rejected;
            cnt->triangles_clipped += j.local[t].triangles_clipped;
            cnt->triangles_visible += j.local[t].triangles_visible;
            cnt->quads += j.local[t].quads;
            cnt->fragments_tested += j.local[t].fragments_tested;
            cnt->fragments_passed += j.local[t].fragments_passed;
            cnt->texture_levels_mask |= j.local[t].texture_levels_mask;
        }
    pthread_mutex_destroy(&j.mu);
    free(j.prims);
    free(j.spans);
    return SWGB_OK;
}

swgb_status oracle_draw(const swgb_pipeline_state *st, const swgb_draw_args *a, int nthreads, swgb_counters *cnt)
{
    fenv_t saved;
    hw_flush_on(&saved);
    const swgb_status s = draw_impl(st, a, nthreads, cnt, NULL, NULL, 0);
    fesetenv(&saved);
    return s;
}

swgb_status oracle_draw_visibility(const swgb_pipeline_state *st, const swgb_draw_args *a, int nthreads, swgb_counters *cnt,
                                   uint32_t *vis, uint32_t *visLen, int visCap)
{
    if(!vis || !visLen || visCap < 1) return SWGB_INVALID_ARG;
    fenv_t saved;
    hw_flush_on(&saved);
    const swgb_status s = draw_impl(st, a, nthreads, cnt, vis, visLen, visCap);
    fesetenv(&saved);
    return s;
}

int oracle_timing_build(void)
{
#ifdef ORACLE_HW_FLUSH
    return 1;
#else
    return 0;
#endif
}

/* ------------------------------------------------------------------------ */
/* Probes                                                                    */
/* ------------------------------------------------------------------------ */

swgb_status oracle_vertex(const swgb_pipeline_state *st, const swgb_draw_args *a, uint32_t k, float *out_f, int32_t *out_i)
{
    ODraw d;
    swgb_status s = prepare(&d, st, a);
    if(s != SWGB_OK) return s;
    OVertex v;
    vertex_shade(&d, vertex_index(&d, k), &v);
    out_f[0] = v.pos.x; out_f[1] = v.pos.y; out_f[2] = v.pos.z; out_f[3] = v.pos.w;
    out_f[4] = v.pz; out_f[5] = v.pw;
    out_i[0] = v.X; out_i[1] = v.Y; out_i[2] = v.clipFlags;
    return SWGB_OK;
}

int oracle_setup(const swgb_pipeline_state *st, const swgb_draw_args *a, uint32_t tri, int32_t *out_i, uint16_t *spans, int max_rows, float *out_f)
{
    ODraw d;
    if(prepare(&d, st, a) != SWGB_OK) return -1;
    OPrim pr;
    memset(&pr, 0, sizeof(pr));
    uint16_t *buf = (uint16_t *)calloc((size_t)8 * d.rows, sizeof(uint16_t));
    if(!buf) return -1;
    for(int q = 0; q < 4; q++)
    {
        pr.left[q] = buf + (size_t)2 * q * d.rows;
        pr.right[q] = pr.left[q] + d.rows;
    }
    int clipped = 0;
    int vis = process_triangle(&d, tri, &pr, NULL, &clipped);
    out_i[0] = vis ? pr.yMin : 0;
    out_i[1] = vis ? pr.yMax : 0;
    out_i[2] = clipped;
    out_i[3] = vis;
    if(vis && spans)
        for(int y = pr.yMin; y < pr.yMax && y - pr.yMin < max_rows; y++)
        {
            spans[2 * (y - pr.yMin) + 0] = pr.left[0][y + 1];
            spans[2 * (y - pr.yMin) + 1] = pr.right[0][y + 1];
        }
    if(vis && out_f)
    {
        out_f[0] = pr.x0; out_f[1] = pr.y0;
        out_f[2] = pr.z.A; out_f[3] = pr.z.B; out_f[4] = pr.z.C;
        out_f[5] = pr.w.A; out_f[6] = pr.w.B; out_f[7] = pr.w.C;
        for(int k = 0; k < d.nv; k++)
        {
            out_f[8 + 3 * k + 0] = pr.V[k].A;
            out_f[8 + 3 * k + 1] = pr.V[k].B;
            out_f[8 + 3 * k + 2] = pr.V[k].C;
        }
    }
    free(buf);
    return vis;
}

/* ------------------------------------------------------------------------ */
/* Routine-level probes matched by the reference's own routines             */
/* (oracle/refjit/refjit_harness.cpp)                                       */
/* ------------------------------------------------------------------------ */

#define ORACLE_VF (6 + MAXV)

int oracle_triangle_inputs(const swgb_pipeline_state *st, const swgb_draw_args *a, uint32_t tri, float *vf, int32_t *vi,
                           float *consts, int32_t *scissor)
{
    ODraw d;
    if(prepare(&d, st, a) != SWGB_OK) return -1;
    uint32_t k[3];
    triangle_positions(st->topology, st->provoking_vertex == 0, tri, k);
    for(int j = 0; j < 3; j++)
    {
        OVertex v;
        memset(&v, 0, sizeof(v));
        vertex_shade(&d, vertex_index(&d, k[j]), &v);
        float *f = vf + j * ORACLE_VF;
        f[0] = v.pos.x; f[1] = v.pos.y; f[2] = v.pos.z; f[3] = v.pos.w;
        f[4] = v.pz; f[5] = v.pw;
        for(int c = 0; c < MAXV; c++) f[6 + c] = c < d.nv ? v.v[c] : 0.0f;
        vi[3 * j + 0] = v.X; vi[3 * j + 1] = v.Y; vi[3 * j + 2] = v.clipFlags;
    }
    consts[0] = d.WxF; consts[1] = d.HxF; consts[2] = d.X0xF; consts[3] = d.Y0xF;
    consts[4] = d.depthRange; consts[5] = d.depthNear;
    scissor[0] = d.sx0; scissor[1] = d.sx1; scissor[2] = d.sy0; scissor[3] = d.sy1;
    return d.nv;
}

int oracle_setup_samples(const swgb_pipeline_state *st, const swgb_draw_args *a, uint32_t tri, int32_t *out_i, uint16_t *spans,
                         int max_rows, float *out_f)
{
    ODraw d;
    if(prepare(&d, st, a) != SWGB_OK) return -1;
    OPrim pr;
    memset(&pr, 0, sizeof(pr));
    uint16_t *buf = (uint16_t *)calloc((size_t)8 * d.rows, sizeof(uint16_t));
    if(!buf) return -1;
    for(int q = 0; q < 4; q++)
    {
        pr.left[q] = buf + (size_t)2 * q * d.rows;
        pr.right[q] = pr.left[q] + d.rows;
    }
    int clipped = 0;
    int vis = process_triangle(&d, tri, &pr, NULL, &clipped);
    out_i[0] = vis ? pr.yMin : 0;
    out_i[1] = vis ? pr.yMax : 0;
    out_i[2] = clipped;
    out_i[3] = vis;
    int rc = 0;
    if(vis && spans)
    {
        int rows = pr.yMax - pr.yMin + 2;
        if(rows > max_rows) rc = -1;
        else
            for(int q = 0; q < d.ms; q++)
                for(int r = 0; r < rows; r++)
                {
                    int y = pr.yMin - 1 + r; /* left/right are indexed [y + 1] */
                    spans[((size_t)q * max_rows + r) * 2 + 0] = pr.left[q][y + 1];
                    spans[((size_t)q * max_rows + r) * 2 + 1] = pr.right[q][y + 1];
                }
    }
    if(vis && out_f)
    {
        out_f[0] = pr.x0; out_f[1] = pr.y0;
        out_f[2] = pr.z.A; out_f[3] = pr.z.B; out_f[4] = pr.z.C;
        out_f[5] = pr.w.A; out_f[6] = pr.w.B; out_f[7] = pr.w.C;
        for(int k = 0; k < d.nv; k++)
        {
            out_f[8 + 3 * k + 0] = pr.V[k].A;
            out_f[8 + 3 * k + 1] = pr.V[k].B;
            out_f[8 + 3 * k + 2] = pr.V[k].C;
        }
        out_f[8 + 3 * d.nv] = pr.zBias;
    }
    free(buf);
    return rc == 0 ? vis : rc;
}
