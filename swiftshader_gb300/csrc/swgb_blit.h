// swgb_blit.h -- launch interface between the C-ABI (swgb_draw.cu) and the
// Blitter kernels (swgb_blit.cu, compiled without flush-to-zero).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/swgb.h"

namespace swgbb {

// Colour formats of the Blitter kernels.
enum { BK_RGBA8 = 0, BK_BGRA8 = 1, BK_RGBA16F = 2, BK_RGBA32F = 3 };

// One generic blit (Blitter::generate's routine state and BlitData, 2D).
struct BlitParams {
    const uint8_t *src;
    uint8_t *dst;
    int64_t sPitch, sSlice, dPitch;
    int srcKind, dstKind;
    int sBytes, dBytes;
    int srcSRGB, dstSRGB;
    int srcSamples;
    int filter;       // bilinear
    int clampToEdge;  // the source region reaches outside the image, or the filter reads at its edge
    int allowSRGB;    // sRGB conversion allowed (filtering, resolving or an encoding change)
    float x0, y0, w, h;
    int x0d, x1d, y0d, y1d;
    int sW, sH;
    int vec16;  // source base and row pitch 16-byte aligned
};

// The byte-averaging 4-sample resolve of an 8-bit image.
struct ResolveParams {
    const uint8_t *src;
    uint8_t *dst;
    int64_t sPitch, sSlice, dPitch;
    int width, height;
    int vec16;  // every row start 16-byte aligned: four pixels per 16-byte access
};

// One clear of an area of every sample plane.
struct ClearParams {
    uint8_t *dst;
    int64_t pitch, slice;
    int x, y;           // the area's origin
    int rows, planes;   // its height; sample planes
    int64_t rowBytes;   // its width in bytes
    int bpp;            // texel size: 1, 2, 4, 8 or 16
    uint32_t dstFormat;
    int dstKind, dstSRGB, normalized;
    float value[4];
    uint32_t stencil;
};

cudaError_t launch_blit(const BlitParams &P, cudaStream_t st);
cudaError_t launch_resolve_bytes(const ResolveParams &R, cudaStream_t st);
cudaError_t launch_clear(const ClearParams &C, cudaStream_t st);

}  // namespace swgbb
