/*
 * TEST INFRASTRUCTURE ONLY -- CPU restatement of the reference's Blitter for
 * the formats of the draw path: clears, multisample resolves and scaled blits
 * (src/Device/Blitter.cpp).  The checker for swgb_clear / swgb_resolve /
 * swgb_blit; never part of the product path.
 *
 * Arithmetic is plain IEEE binary32 with subnormals kept: the reference runs
 * blit routines on its queue thread, which does not set FTZ/DAZ (only marl
 * worker threads do, src/System/SwiftConfig.cpp:136-139).  Built with
 * -ffp-contract=off so that every multiply and add rounds on its own, as the
 * JIT-emitted routine's separate fmul / fadd instructions do; fmaf() stands
 * for MulAdd where the reference writes it.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../include/swgb.h"

enum { K_RGBA8 = 0, K_BGRA8 = 1, K_RGBA16F = 2, K_RGBA32F = 3 };

typedef struct {
    int colour, kind, srgb, bytes;
} bfmt;

static bfmt fmt_of(uint32_t f)
{
    switch(f)
    {
    case SWGB_FORMAT_R8G8B8A8_UNORM: return (bfmt){1, K_RGBA8, 0, 4};
    case SWGB_FORMAT_R8G8B8A8_SRGB: return (bfmt){1, K_RGBA8, 1, 4};
    case SWGB_FORMAT_B8G8R8A8_UNORM: return (bfmt){1, K_BGRA8, 0, 4};
    case SWGB_FORMAT_B8G8R8A8_SRGB: return (bfmt){1, K_BGRA8, 1, 4};
    case SWGB_FORMAT_R16G16B16A16_SFLOAT: return (bfmt){1, K_RGBA16F, 0, 8};
    case SWGB_FORMAT_R32G32B32A32_SFLOAT: return (bfmt){1, K_RGBA32F, 0, 16};
    case SWGB_FORMAT_D32_SFLOAT: return (bfmt){0, -1, 0, 4};
    case SWGB_FORMAT_D16_UNORM: return (bfmt){0, -1, 0, 2};
    case SWGB_FORMAT_S8_UINT: return (bfmt){0, -1, 0, 1};
    default: return (bfmt){0, -1, 0, 0};
    }
}

static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static float rmin(float x, float y) { return x < y ? x : y; } /* Min: minps */
static float rmax(float x, float y) { return x > y ? x : y; } /* Max: maxps */
/* RoundInt (cvtps2dq) and Int(Float) (cvttps2dq): 0x80000000 when out of range */
static int32_t round_int(float x) { return (x >= -2147483648.0f && x < 2147483648.0f) ? (int32_t)nearbyintf(x) : INT32_MIN; }
static int32_t trunc_int(float x) { return (x >= -2147483648.0f && x < 2147483648.0f) ? (int32_t)x : INT32_MIN; }

/* Reactor's Float(Half) (src/Reactor/Reactor.cpp:3787-3815) */
static float half_to_float(uint32_t h)
{
    int32_t s = (int32_t)((h >> 15) & 1u), e = (int32_t)((h >> 10) & 0x1Fu), m = (int32_t)(h & 0x3FFu);
    uint32_t r = (uint32_t)s << 31;
    if(e == 0)
    {
        if(m != 0)
        {
            while((m & 0x400) == 0)
            {
                m <<= 1;
                e -= 1;
            }
            r |= (uint32_t)(((e + (127 - 15) + 1) << 23) | ((m & ~0x400) << 13));
        }
    }
    else
        r |= (uint32_t)(((e + (127 - 15)) << 23) | (m << 13));
    return u2f(r);
}

/* Reactor's Half(Float) (src/Reactor/Reactor.cpp:3744-3770) */
static uint32_t float_to_half(float f)
{
    uint32_t x = f2u(f), a = x & 0x7FFFFFFFu, h = (x & 0x80000000u) >> 16;
    if(a > 0x47FFEFFFu)
        h |= 0x7FFFu;
    else if(a < 0x38800000u)
    {
        int32_t mant = (int32_t)((a & 0x007FFFFFu) | 0x00800000u), e = 113 - (int32_t)(a >> 23);
        uint32_t a2 = e < 24 ? (uint32_t)(mant >> e) : 0u;
        h |= ((a2 + 0x00000FFFu + ((a2 >> 13) & 1u)) >> 13) & 0xFFFFu;
    }
    else
        h |= ((a + 0xC8000000u + 0x00000FFFu + ((a >> 13) & 1u)) >> 13) & 0xFFFFu;
    return h & 0xFFFFu;
}

/* Pow<Mediump> and the sRGB transfer functions (src/Pipeline/ShaderCore.cpp:
 * 336-386,406-470,472-477,914-930), IEEE arithmetic. */
static float log2_mp(float x)
{
    const int32_t im = (int32_t)f2u(x);
    float y = fmaf((float)im, 1.0f / (1 << 23), -127.0f);
    if(im == 0x7F800000) y = u2f(f2u(y) | 0x7F800000u);
    const float m = (float)(im & 0x007FFFFF);
    const float f = fmaf(fmaf(2.8017103e-22f, m, -8.373131e-15f), m, 5.0615534e-8f);
    return fmaf(f, m, y);
}
static float exp2_mp(float x)
{
    float x0 = rmin(x, 128.0f);
    x0 = rmax(x0, u2f(0xC2FDFFFFu));
    const float f = x0 - floorf(x0);
    const float r = fmaf(fmaf(7.8145574e-2f, f, 2.2617357e-1f), f, -3.0444314e-1f);
    const float y = fmaf(r, f, x0);
    return u2f((uint32_t)trunc_int(fmaf((float)(1 << 23), y, (float)(127 << 23))));
}
static float pow_mp(float x, float y) { return exp2_mp(log2_mp(x) * y); }
static float lin_to_srgb(float c)
{
    const float lc = c * 12.92f, ec = fmaf(1.055f, pow_mp(c, 1.0f / 2.4f), -0.055f);
    return c < 0.0031308f ? lc : ec;
}
static float srgb_to_lin(float c)
{
    const float lc = c * (1.0f / 12.92f), ec = pow_mp(fmaf(c, 1.0f / 1.055f, 0.055f / 1.055f), 2.4f);
    return c < 0.04045f ? lc : ec;
}

/* readFloat4 (Blitter.cpp:312-550) */
static void read_texel(const uint8_t *p, int kind, float c[4])
{
    if(kind == K_RGBA8 || kind == K_BGRA8)
    {
        for(int k = 0; k < 4; k++) c[k] = (float)p[k];
        if(kind == K_BGRA8)
        {
            const float t = c[0];
            c[0] = c[2];
            c[2] = t;
        }
    }
    else if(kind == K_RGBA16F)
        for(int k = 0; k < 4; k++) c[k] = half_to_float((uint32_t)p[2 * k] | ((uint32_t)p[2 * k + 1] << 8));
    else
        memcpy(c, p, 16);
}

/* RoundShort4 + PackUnsigned (Reactor.cpp:1947-1951) */
static uint8_t pack_unorm8(float c)
{
    int32_t r = round_int(c);
    r = r < -32768 ? -32768 : (r > 32767 ? 32767 : r);
    return (uint8_t)(r < 0 ? 0 : (r > 255 ? 255 : r));
}

/* write (Blitter.cpp:553-1180), all components */
static void write_texel(uint8_t *p, int kind, const float c[4])
{
    if(kind == K_RGBA8)
        for(int k = 0; k < 4; k++) p[k] = pack_unorm8(c[k]);
    else if(kind == K_BGRA8)
    {
        p[0] = pack_unorm8(c[2]);
        p[1] = pack_unorm8(c[1]);
        p[2] = pack_unorm8(c[0]);
        p[3] = pack_unorm8(c[3]);
    }
    else if(kind == K_RGBA16F)
        for(int k = 0; k < 4; k++)
        {
            const uint32_t h = float_to_half(c[k]);
            p[2 * k] = (uint8_t)h;
            p[2 * k + 1] = (uint8_t)(h >> 8);
        }
    else
        memcpy(p, c, 16);
}

static int is_float(int kind) { return kind == K_RGBA16F || kind == K_RGBA32F; }
static int is_unorm8(int kind) { return kind == K_RGBA8 || kind == K_BGRA8; }

/* ApplyScaleAndClamp (Blitter.cpp:1427-1485) for these formats */
static void scale_and_clamp(float v[4], int sk, int ssrgb, int dk, int dsrgb, int allow, int preScaled)
{
    const float unscale = is_unorm8(sk) ? 255.0f : 1.0f, scale = is_unorm8(dk) ? 255.0f : 1.0f;
    if(allow && ((ssrgb && !preScaled) || dsrgb))
    {
        const float m = preScaled ? 1.0f / scale : 1.0f / unscale;
        for(int k = 0; k < 4; k++) v[k] = v[k] * m;
        for(int k = 0; k < 3; k++) v[k] = (ssrgb && !preScaled) ? srgb_to_lin(v[k]) : lin_to_srgb(v[k]);
        for(int k = 0; k < 4; k++) v[k] = v[k] * scale;
    }
    else if(unscale != scale)
        for(int k = 0; k < 4; k++) v[k] = v[k] * (scale / unscale);
    if(is_float(sk) && !is_float(dk))
        for(int k = 0; k < 4; k++) v[k] = rmax(rmin(v[k], scale), 0.0f);
    if(is_float(sk) && is_unorm8(dk))
        for(int k = 0; k < 4; k++) v[k] = rmax(v[k], 0.0f);
}

typedef struct {
    const uint8_t *src;
    int64_t sPitch, sSlice;
    int sk, dk, ssrgb, dsrgb, sBytes, samples, filter, clampToEdge, allow;
    int sW, sH;
} bstate;

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Blitter::sample (Blitter.cpp:1497-1657), 2D */
static void sample(const bstate *S, float x, float y, float out[4])
{
    const int conv = S->allow && S->ssrgb;
    int preScaled = 0;
    float c[4];
    if(!S->filter)
    {
        int X = trunc_int(x), Y = trunc_int(y);
        if(S->clampToEdge)
        {
            X = clampi(X, 0, S->sW - 1);
            Y = clampi(Y, 0, S->sH - 1);
        }
        X = clampi(X, 0, S->sW - 1);
        Y = clampi(Y, 0, S->sH - 1);
        const uint8_t *s = S->src + (int64_t)Y * S->sPitch + (int64_t)X * S->sBytes;
        read_texel(s, S->sk, c);
        if(S->samples > 1)
        {
            if(conv)
            {
                scale_and_clamp(c, S->sk, S->ssrgb, S->dk, S->dsrgb, S->allow, 0);
                preScaled = 1;
            }
            float acc[4] = {c[0], c[1], c[2], c[3]};
            for(int q = 1; q < S->samples; q++)
            {
                s += S->sSlice;
                read_texel(s, S->sk, c);
                if(conv) scale_and_clamp(c, S->sk, S->ssrgb, S->dk, S->dsrgb, S->allow, 0);
                for(int k = 0; k < 4; k++) acc[k] = acc[k] + c[k];
            }
            for(int k = 0; k < 4; k++) c[k] = acc[k] * (1.0f / (float)S->samples);
        }
    }
    else
    {
        float X = x, Y = y;
        if(S->clampToEdge)
        {
            X = rmin(rmax(x, 0.5f), (float)S->sW - 0.5f);
            Y = rmin(rmax(y, 0.5f), (float)S->sH - 0.5f);
        }
        const float x0 = X - 0.5f, y0 = Y - 0.5f;
        int X0 = trunc_int(x0), Y0 = trunc_int(y0);
        X0 = X0 > 0 ? X0 : 0;
        Y0 = Y0 > 0 ? Y0 : 0;
        int X1 = X0 + 1, Y1 = Y0 + 1;
        X1 = X1 >= S->sW ? X0 : X1;
        Y1 = Y1 >= S->sH ? Y0 : Y1;
        const int xs[2] = {clampi(X0, 0, S->sW - 1), clampi(X1, 0, S->sW - 1)};
        const int ys[2] = {clampi(Y0, 0, S->sH - 1), clampi(Y1, 0, S->sH - 1)};
        float t[4][4]; /* c00, c01, c10, c11 */
        for(int k = 0; k < 4; k++)
        {
            read_texel(S->src + (int64_t)ys[k >> 1] * S->sPitch + (int64_t)xs[k & 1] * S->sBytes, S->sk, t[k]);
            if(conv) scale_and_clamp(t[k], S->sk, S->ssrgb, S->dk, S->dsrgb, S->allow, 0);
        }
        if(conv) preScaled = 1;
        const float fx = x0 - (float)X0, fy = y0 - (float)Y0, ix = 1.0f - fx, iy = 1.0f - fy;
        for(int k = 0; k < 4; k++) c[k] = (t[0][k] * ix + t[1][k] * fx) * iy + (t[2][k] * ix + t[3][k] * fx) * fy;
    }
    scale_and_clamp(c, S->sk, S->ssrgb, S->dk, S->dsrgb, S->allow, preScaled);
    memcpy(out, c, 16);
}

static int blit_region(const swgb_image *src, const swgb_image *dst, swgb_blit_region r, int filter)
{
    const bfmt sf = fmt_of(src->format), df = fmt_of(dst->format);
    if(!sf.colour || !df.colour) return SWGB_UNSUPPORTED_STATE;
    if(r.dst[0] > r.dst[2])
    {
        int32_t t = r.src[0]; r.src[0] = r.src[2]; r.src[2] = t;
        t = r.dst[0]; r.dst[0] = r.dst[2]; r.dst[2] = t;
    }
    if(r.dst[1] > r.dst[3])
    {
        int32_t t = r.src[1]; r.src[1] = r.src[3]; r.src[3] = t;
        t = r.dst[1]; r.dst[1] = r.dst[3]; r.dst[3] = t;
    }
    if(r.dst[0] < 0 || r.dst[1] < 0 || (uint32_t)r.dst[2] > dst->width || (uint32_t)r.dst[3] > dst->height) return SWGB_INVALID_ARG;
    if(r.dst[0] == r.dst[2] || r.dst[1] == r.dst[3]) return SWGB_OK;
    /* Blitter::blit (Blitter.cpp:1820-1895) */
    const float wr = (float)(r.src[2] - r.src[0]) / (float)(r.dst[2] - r.dst[0]);
    const float hr = (float)(r.src[3] - r.src[1]) / (float)(r.dst[3] - r.dst[1]);
    const float x0 = (float)r.src[0] + (0.5f - (float)r.dst[0]) * wr;
    const float y0 = (float)r.src[1] + (0.5f - (float)r.dst[1]) * hr;
    bstate S;
    S.src = (const uint8_t *)src->data;
    S.sPitch = (int64_t)src->pitch_bytes;
    S.sSlice = (int64_t)src->slice_bytes;
    S.sk = sf.kind;
    S.dk = df.kind;
    S.ssrgb = sf.srgb;
    S.dsrgb = df.srgb;
    S.sBytes = sf.bytes;
    S.samples = (int)src->samples;
    S.filter = filter;
    S.allow = filter || src->samples > 1 || sf.srgb != df.srgb;
    S.clampToEdge = r.src[0] < 0 || r.src[1] < 0 || (uint32_t)r.src[2] > src->width || (uint32_t)r.src[3] > src->height ||
                    (filter && (x0 < 0.5f || y0 < 0.5f));
    S.sW = (int)src->width;
    S.sH = (int)src->height;
    uint8_t *d = (uint8_t *)dst->data;
    for(int j = r.dst[1]; j < r.dst[3]; j++)
    {
        const float y = y0 + (float)j * hr;
        for(int i = r.dst[0]; i < r.dst[2]; i++)
        {
            const float x = x0 + (float)i * wr;
            float c[4];
            sample(&S, x, y, c);
            write_texel(d + (int64_t)j * (int64_t)dst->pitch_bytes + (int64_t)i * df.bytes, df.kind, c);
        }
    }
    return SWGB_OK;
}

int oracle_blit(const swgb_image *src, const swgb_image *dst, const swgb_blit_region *region, uint32_t filter)
{
    if(src->samples != 1 || dst->samples != 1) return SWGB_INVALID_ARG;
    return blit_region(src, dst, *region, filter == SWGB_FILTER_LINEAR);
}

/* averageByte4 (Blitter.cpp:2074-2077) */
static uint32_t avg_byte4(uint32_t x, uint32_t y) { return (x & y) + (((x ^ y) >> 1) & 0x7F7F7F7Fu) + ((x ^ y) & 0x01010101u); }

int oracle_resolve(const swgb_image *src, const swgb_image *dst, const swgb_resolve_region *region)
{
    if(src->format != dst->format || !fmt_of(src->format).colour || src->samples != 4 || dst->samples != 1) return SWGB_INVALID_ARG;
    swgb_resolve_region r = region ? *region : (swgb_resolve_region){0, 0, 0, 0, src->width, src->height};
    const int whole = r.src_x == 0 && r.src_y == 0 && r.dst_x == 0 && r.dst_y == 0 && r.width == src->width &&
                      r.height == src->height && src->width == dst->width && src->height == dst->height;
    if(whole && (src->format == SWGB_FORMAT_R8G8B8A8_UNORM || src->format == SWGB_FORMAT_B8G8R8A8_UNORM))
    {
        /* fastResolve (Blitter.cpp:2079-2205) */
        for(uint32_t y = 0; y < r.height; y++)
            for(uint32_t x = 0; x < r.width; x++)
            {
                const uint8_t *s = (const uint8_t *)src->data + (size_t)y * src->pitch_bytes + (size_t)x * 4;
                uint32_t c[4];
                for(int q = 0; q < 4; q++) memcpy(&c[q], s + (size_t)q * src->slice_bytes, 4);
                const uint32_t o = avg_byte4(avg_byte4(c[0], c[1]), avg_byte4(c[2], c[3]));
                memcpy((uint8_t *)dst->data + (size_t)y * dst->pitch_bytes + (size_t)x * 4, &o, 4);
            }
        return SWGB_OK;
    }
    swgb_blit_region b = {{r.src_x, r.src_y, r.src_x + (int32_t)r.width, r.src_y + (int32_t)r.height},
                          {r.dst_x, r.dst_y, r.dst_x + (int32_t)r.width, r.dst_y + (int32_t)r.height}};
    return blit_region(src, dst, b, 0);
}

/* Blitter::clear (Blitter.cpp:55-168) and fastClear (:170-300) */
int oracle_clear(const void *value, uint32_t value_format, const swgb_image *dst, const swgb_rect *area)
{
    const bfmt f = fmt_of(dst->format);
    if(f.bytes == 0) return SWGB_UNSUPPORTED_STATE;
    swgb_rect a = area ? *area : (swgb_rect){0, 0, dst->width, dst->height};
    float v[4] = {0, 0, 0, 0};
    uint32_t stencil = 0;
    if(value_format == SWGB_FORMAT_S8_UINT)
        memcpy(&stencil, value, 4);
    else
        memcpy(v, value, value_format == SWGB_FORMAT_D32_SFLOAT ? 4 : 16);
    const int normalized = (f.colour && !is_float(f.kind)) || dst->format == SWGB_FORMAT_D16_UNORM;
    if(normalized)
        for(int k = 0; k < 4; k++)
        {
            if(v[k] < 0.0f) v[k] = 0.0f;
            if(v[k] > 1.0f) v[k] = 1.0f;
        }
    uint8_t t[16] = {0};
    switch(dst->format)
    {
    case SWGB_FORMAT_R8G8B8A8_UNORM:
    case SWGB_FORMAT_B8G8R8A8_UNORM:
    {
        uint8_t c[4];
        for(int k = 0; k < 4; k++) c[k] = (uint8_t)(uint32_t)(255 * v[k] + 0.5f);
        if(dst->format == SWGB_FORMAT_R8G8B8A8_UNORM)
            memcpy(t, c, 4);
        else
        {
            t[0] = c[2];
            t[1] = c[1];
            t[2] = c[0];
            t[3] = c[3];
        }
        break;
    }
    case SWGB_FORMAT_D32_SFLOAT: memcpy(t, value, 4); break;
    case SWGB_FORMAT_S8_UINT: t[0] = (uint8_t)stencil; break;
    case SWGB_FORMAT_D16_UNORM:
    {
        float x = v[0] * 65535.0f;
        x = rmax(rmin(x, 65535.0f), 0.0f);
        const uint32_t h = (uint32_t)round_int(x) & 0xFFFFu;
        t[0] = (uint8_t)h;
        t[1] = (uint8_t)(h >> 8);
        break;
    }
    default:
        scale_and_clamp(v, K_RGBA32F, 0, f.kind, f.srgb, 1, 0);
        write_texel(t, f.kind, v);
        break;
    }
    for(uint32_t q = 0; q < dst->samples; q++)
        for(uint32_t y = 0; y < a.height; y++)
        {
            uint8_t *row = (uint8_t *)dst->data + (size_t)q * dst->slice_bytes + (size_t)(a.y + (int32_t)y) * dst->pitch_bytes +
                           (size_t)a.x * f.bytes;
            for(uint32_t x = 0; x < a.width; x++) memcpy(row + (size_t)x * f.bytes, t, (size_t)f.bytes);
        }
    return SWGB_OK;
}
