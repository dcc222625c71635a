// swgb_draw.cu -- host side and C-ABI of the GB300 (sm_103a) draw hot path,
// plus the vertex, setup and adjoint kernels (device code in swgb_kernels.cuh;
// the raster kernel variants are compiled from swgb_raster.cu).
//
// Pipeline per draw (all on the context's stream, no host round trip):
//   k_vertex  : one thread per vertex -- fetch, fixed VS (MVP), clip flags,
//               projection + viewport snap.  Post-transform vertices stay in
//               HBM/L2 like the reference's vertex cache
//               (src/Pipeline/VertexRoutine.cpp:43-87,116-154,570-707).
//   k_setup   : one thread per triangle, 256-triangle blocks -- trivial
//               reject, homogeneous clipping, cull, sub-pixel polygon, y range,
//               the reference's integer DDA span rows, empty-row trimming,
//               pixel boxes; block-reduced chunk and super-chunk boxes drive
//               the binning (src/Device/Renderer.cpp:733-776,
//               src/Device/Clipper.cpp, src/Pipeline/SetupRoutine.cpp:36-621).
//   k_raster  : persistent warps, one screen bin (16x16, 32x16 or 32x32
//               pixels) per warp from an atomic queue -- depth and colour of
//               the bin staged in shared memory with 16-byte accesses; the
//               super-chunk, chunk and triangle boxes tested in primitive order
//               with warp ballots; per batch of 32 triangles the span rows and
//               plane equations staged, triangles behind the bin's depth bound
//               rejected whole, quads expanded and masked, early depth
//               rejection, per-pixel shading (interpolation, SamplerCore
//               filtering, fixed FS) and an ordered per-pixel resolve of depth
//               test, blend and colour write; the bin written back with 16-byte
//               stores (src/Device/QuadRasterizer.cpp:36-250,
//               src/Pipeline/PixelRoutine.cpp:97-358,494-739,1225-2700,
//               src/Pipeline/PixelProgram.cpp:138-364,
//               src/Pipeline/SamplerCore.cpp).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "swgb_blit.h"
#include "swgb_kernels.cuh"

using namespace swgbk;

// ==========================================================================
// Host side: context, state baking, C-ABI
// ==========================================================================

struct swgb_ctx {
    int device;
    cudaStream_t stream;
    cudaStream_t side;            // second stream: k_bin_order beside k_bin_list
    cudaEvent_t sideFork, sideJoin;
    bool ownStream;
    float4 *ptv;
    size_t ptvCap;
    short4 *triBox;
    size_t triBoxCap;
    TriInfo *triInfo;
    size_t triInfoCap;
    float4 *planes;
    size_t planesCap;
    uint32_t *spans;
    size_t spansCap;
    unsigned long long *spanCount;
    uint64_t spanRowsLimit;
    short4 *chunkBox;
    size_t chunkCap;
    int4 *superBox;
    size_t superCap;
    int2 *poly;
    size_t polyCap;
    uint32_t *polyCount;
    unsigned int *binQueue;
    uint16_t *srgbLut;     // sRGBtoLinearFF_FF00 on the device (256 entries)
    uint32_t *restart;     // primitive restart: per-position segment starts, then per-block carries
    size_t restartCap;
    int *binDiff;          // bin order of single draws: difference array, then the first chunk per bin
    size_t binDiffCap;
    uint32_t *binOrder;
    size_t binOrderCap;
    uint32_t *binList;        // candidate lists of single draws' bins, then their counts
    size_t binListCap;
    uint32_t binListPerBin;   // entries per bin list (0: no lists)
    uint32_t binListMinTris;  // draws with fewer triangles walk their bins in k_raster
    bool binOrderAttr;
    int rasterBlocks[NRASTER];  // persistent raster grid per kernel variant: SMs x resident blocks per SM
    swgb_raster_config rasterConfig;  // bin shape and depth rejection of single-sample draws
    unsigned long long *counters;
    int *error;
    uint64_t launches;
    bool rasterAttr;
    bool timing;
    uint32_t timingKinds;  // bit k: launches of kind k get an event pair while timing
    std::vector<cudaEvent_t> *evFree;           // recycled events
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> *evPairs;
    struct BatchState *batch;                   // batched-draw scratch, descriptors and graphs
    bool adjAttr;
    int adjBlocks[2];      // persistent adjoint grid: 1 and 4 samples
    uint8_t *adjScratch;   // one region per adjoint warp of the larger grid
    double *ptv64;         // adjoint: fp64 clip coordinates per vertex
    size_t ptv64Cap;
};

namespace {

thread_local std::string g_error;

swgb_status set_error(swgb_status s, const char *msg)
{
    g_error = msg;
    return s;
}

swgb_status cuda_check(cudaError_t e, const char *what)
{
    if(e == cudaSuccess) return SWGB_OK;
    g_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SWGB_OOM : SWGB_DEVICE_ERROR;
}

template<typename T>
swgb_status ensure(T *&ptr, size_t &cap, size_t need, const char *what)
{
    if(need <= cap && ptr) return SWGB_OK;
    if(ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t n = need < 1 ? 1 : need;
    swgb_status s = cuda_check(cudaMalloc((void **)&ptr, n * sizeof(T)), what);
    if(s != SWGB_OK) return s;
    cap = n;
    return SWGB_OK;
}

uint32_t simplify_op(uint32_t op, uint32_t sf, uint32_t df)
{
    // vk::FragmentOutputInterfaceState::blendOperation (src/Device/Context.cpp:1181-1270)
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
        if(sf == SWGB_BLEND_ZERO) return OP_ZERO_EXT;  // UNORM target: negative clamps to zero
        if(sf == SWGB_BLEND_ONE && df == SWGB_BLEND_ZERO) return OP_SRC_EXT;
        break;
    case SWGB_BLEND_OP_REVERSE_SUBTRACT:
        if(sf == SWGB_BLEND_ZERO)
        {
            if(df == SWGB_BLEND_ZERO) return OP_ZERO_EXT;
            if(df == SWGB_BLEND_ONE) return OP_DST_EXT;
        }
        break;
    default: break;
    }
    return op;
}

// Validates the state and bakes DrawParams (Renderer::draw, src/Device/Renderer.cpp:183-490).
// Bins of shape bw x bh (powers of two) over the draw's scissor.
void set_bins(DrawParams &D, int bw, int bh)
{
    D.binW = bw;
    D.binH = bh;
    D.binX0 = D.sx0 & ~(bw - 1);
    D.binY0 = D.sy0 & ~(bh - 1);
    D.binsX = (D.sx1 - D.binX0 + bw - 1) / bw;
    D.binsY = (D.sy1 - D.binY0 + bh - 1) / bh;
}

// sRGBtoLinearFF_FF00, the table the reference's sampler decodes 8-bit sRGB
// texels with (src/Pipeline/Constants.cpp:273-276, sw::sRGBtoLinear
// src/System/Math.hpp:326-336): linear value with 0xFF00 = 1.0, computed on
// the host at start-up as the reference does.
void srgb_table(uint16_t out[256])
{
    for(int i = 0; i < 256; i++)
    {
        const float c = (float)i / 0xFF;
        const float lin = c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
        out[i] = (uint16_t)(lin * 0xFF00 + 0.5f);
    }
}

swgb_status bake(const swgb_pipeline_state *st, const swgb_draw_args *a, DrawParams &D)
{
    memset(&D, 0, sizeof(D));
    if(st->precision_profile != SWGB_PRECISION_CMAKE) return set_error(SWGB_UNSUPPORTED_STATE, "only the CMake precision profile is implemented");
    if(st->topology != SWGB_TOPOLOGY_TRIANGLE_LIST && st->topology != SWGB_TOPOLOGY_TRIANGLE_STRIP &&
       st->topology != SWGB_TOPOLOGY_TRIANGLE_FAN)
        return set_error(SWGB_UNSUPPORTED_STATE, "topology (triangle list, strip or fan)");
    if(st->sample_count != 1 && st->sample_count != 4) return set_error(SWGB_UNSUPPORTED_STATE, "sample_count (1 or 4)");
    if(st->vertex_shader != SWGB_VS_MVP_PASSTHROUGH) return set_error(SWGB_UNSUPPORTED_STATE, "vertex_shader");
    if(st->fragment_shader != SWGB_FS_VCOLOR && st->fragment_shader != SWGB_FS_TEX_X_VCOLOR) return set_error(SWGB_UNSUPPORTED_STATE, "fragment_shader");
    if(st->depth_clamp_enable) return set_error(SWGB_UNSUPPORTED_STATE, "depth clamp");
    if(st->color_format != SWGB_FORMAT_R8G8B8A8_UNORM && st->color_format != SWGB_FORMAT_B8G8R8A8_UNORM &&
       st->color_format != SWGB_FORMAT_R8G8B8A8_SRGB && st->color_format != SWGB_FORMAT_B8G8R8A8_SRGB &&
       st->color_format != SWGB_FORMAT_R16G16B16A16_SFLOAT && st->color_format != SWGB_FORMAT_R32G32B32A32_SFLOAT)
        return set_error(SWGB_UNSUPPORTED_STATE, "color_format");
    if(st->depth_format != SWGB_FORMAT_UNDEFINED && st->depth_format != SWGB_FORMAT_D32_SFLOAT && st->depth_format != SWGB_FORMAT_D16_UNORM)
        return set_error(SWGB_UNSUPPORTED_STATE, "depth_format");
    if(!st->color) return set_error(SWGB_INVALID_ARG, "color attachment is null");
    if(st->attrib_count < 1 || st->attrib_count > SWGB_MAX_ATTRIBS) return set_error(SWGB_INVALID_ARG, "attrib_count");
    if(st->color_blend_op > SWGB_BLEND_OP_MAX || st->alpha_blend_op > SWGB_BLEND_OP_MAX) return set_error(SWGB_UNSUPPORTED_STATE, "blend op");
    if(st->framebuffer_width > 16384 || st->framebuffer_height > 16384) return set_error(SWGB_UNSUPPORTED_STATE, "framebuffer larger than 16384");
    D.nattr = (int)st->attrib_count;
    D.nv = 0;
    for(int i = 0; i < D.nattr; i++)
    {
        const swgb_vertex_attrib &at = st->attribs[i];
        if(at.binding >= SWGB_MAX_ATTRIBS || !st->bindings[at.binding].buffer) return set_error(SWGB_INVALID_ARG, "vertex binding");
        if(at.format != SWGB_FORMAT_R32G32B32A32_SFLOAT && at.format != SWGB_FORMAT_R32G32_SFLOAT) return set_error(SWGB_UNSUPPORTED_STATE, "vertex format");
        D.vbuf[i] = (const uint8_t *)st->bindings[at.binding].buffer;
        D.vstride[i] = st->bindings[at.binding].stride;
        D.voff[i] = at.offset;
        D.vcomp[i] = at.format == SWGB_FORMAT_R32G32_SFLOAT ? 2 : 4;
        if(i > 0) D.nv += (int)D.vcomp[i];
    }
    if(D.nv > PLANE_V) return set_error(SWGB_UNSUPPORTED_STATE, "too many varyings");
    D.planeVec4 = (8 + 3 * D.nv + 3) / 4;  // grown to the zBias plane below when the draw has depth bias
    if(D.nattr < 2 || D.vcomp[1] != 4) return set_error(SWGB_INVALID_ARG, "the fixed FS reads a vec4 colour at location 0");
    D.fs = (int)st->fragment_shader;
    if(D.fs == SWGB_FS_TEX_X_VCOLOR && (D.nattr < 3 || D.nv < 6)) return set_error(SWGB_INVALID_ARG, "textured FS needs a uv varying");
    memcpy(D.mvp, st->mvp, sizeof(D.mvp));

    if(st->provoking_vertex > 1) return set_error(SWGB_INVALID_ARG, "provoking_vertex (0 first, 1 last)");
    D.provokingLast = st->provoking_vertex == 1;
    D.count = a->count;
    D.indexType = a->index_type;
    D.indices = a->indices;
    D.firstVertex = a->first_vertex;
    D.baseVertex = a->base_vertex;
    D.topology = st->topology;
    if(a->index_type == SWGB_INDEX_TYPE_NONE)
        D.vertexCount = st->topology == SWGB_TOPOLOGY_TRIANGLE_LIST ? 3u * a->count : a->count + 2u;
    else
    {
        if(a->index_type != SWGB_INDEX_TYPE_UINT16 && a->index_type != SWGB_INDEX_TYPE_UINT32 && a->index_type != SWGB_INDEX_TYPE_UINT8)
            return set_error(SWGB_INVALID_ARG, "index_type");
        if(!a->indices) return set_error(SWGB_INVALID_ARG, "indices");
        if(a->vertex_count == 0) return set_error(SWGB_INVALID_ARG, "indexed draws need vertex_count");
        D.vertexCount = a->vertex_count;
        if(a->restart_index_count)
        {
            // triangle slots are index positions; k_restart_* find the sub-draws
            D.restart = 1;
            D.count = a->restart_index_count;
            D.restartValue = a->index_type == SWGB_INDEX_TYPE_UINT8 ? 0xFFu : (a->index_type == SWGB_INDEX_TYPE_UINT16 ? 0xFFFFu : 0xFFFFFFFFu);
        }
    }

    // Viewport and scissor (Renderer.cpp:300-345)
    float W = 0.5f * st->viewport_width, H = 0.5f * st->viewport_height;
    float X0 = st->viewport_x + W, Y0 = st->viewport_y + H;
    D.WxF = W * 256.0f;
    D.HxF = H * 256.0f;
    D.X0xF = X0 * 256.0f - 128.0f;
    D.Y0xF = Y0 * 256.0f - 128.0f;
    D.depthRange = st->viewport_max_depth - st->viewport_min_depth;
    D.depthNear = st->viewport_min_depth;
    int rx0 = a->render_area_x, ry0 = a->render_area_y;
    int rx1 = rx0 + (int)a->render_area_width, ry1 = ry0 + (int)a->render_area_height;
    auto clampi = [](int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); };
    D.sx0 = clampi(st->scissor_x, rx0, rx1);
    D.sx1 = clampi(st->scissor_x + (int)st->scissor_width, rx0, rx1);
    D.sy0 = clampi(st->scissor_y, ry0, ry1);
    D.sy1 = clampi(st->scissor_y + (int)st->scissor_height, ry0, ry1);
    if(D.sx0 < 0 || D.sy0 < 0 || D.sx1 > (int)st->framebuffer_width || D.sy1 > (int)st->framebuffer_height)
        return set_error(SWGB_INVALID_ARG, "render area outside the framebuffer");
    D.depthClip = st->depth_clip_enable ? 1 : 0;
    D.cullMode = st->cull_mode;
    D.frontFace = st->front_face;

    D.depthTest = st->depth && st->depth_test_enable;
    D.depthWrite = D.depthTest && st->depth_write_enable;
    // depth bias: a NaN clamp counts as 0 (Context.cpp:650-661)
    D.biasConstant = st->depth_bias_constant;
    D.biasSlope = st->depth_bias_slope;
    D.biasClamp = st->depth_bias_clamp == st->depth_bias_clamp ? st->depth_bias_clamp : 0.0f;
    D.depthBias = D.depthTest && (D.biasConstant != 0.0f || D.biasSlope != 0.0f);
    D.depthBounds = st->depth && st->depth_bounds_test_enable;
    D.minBounds = st->min_depth_bounds;
    D.maxBounds = st->max_depth_bounds;
    // stencil (FragmentState::stencilActive and the stencil op states)
    D.stencilTest = st->stencil && st->stencil_test_enable;
    D.earlyDepthOK = 1;
    if(D.stencilTest)
    {
        const swgb_stencil_op_state *ss[2] = {&st->front, &st->back};
        for(int f = 0; f < 2; f++)
        {
            if(ss[f]->fail_op > SWGB_STENCIL_OP_DECREMENT_AND_WRAP || ss[f]->pass_op > SWGB_STENCIL_OP_DECREMENT_AND_WRAP ||
               ss[f]->depth_fail_op > SWGB_STENCIL_OP_DECREMENT_AND_WRAP || ss[f]->compare_op > SWGB_COMPARE_ALWAYS)
                return set_error(SWGB_INVALID_ARG, "stencil op state");
            D.sFailOp[f] = ss[f]->fail_op;
            D.sPassOp[f] = ss[f]->pass_op;
            D.sDepthFailOp[f] = ss[f]->depth_fail_op;
            D.sCompareOp[f] = ss[f]->compare_op;
            D.sCompareMask[f] = ss[f]->compare_mask & 0xFFu;
            D.sWriteMask[f] = ss[f]->write_mask & 0xFFu;
            D.sReference[f] = ss[f]->reference & 0xFFu;
            const bool ops = D.sFailOp[f] != SWGB_STENCIL_OP_KEEP || D.sPassOp[f] != SWGB_STENCIL_OP_KEEP ||
                             D.sDepthFailOp[f] != SWGB_STENCIL_OP_KEEP;
            if(ops && D.sWriteMask[f]) D.stencilWrite = 1;
            // a depth-failing fragment must still update the stencil: no early rejection
            if(D.sWriteMask[f] && (D.sFailOp[f] != SWGB_STENCIL_OP_KEEP || D.sDepthFailOp[f] != SWGB_STENCIL_OP_KEEP)) D.earlyDepthOK = 0;
        }
        D.stencil = (uint8_t *)st->stencil;
        D.stencilPitch = st->stencil_pitch_bytes;
        D.stencilSlice = st->stencil_slice_bytes;
    }
    if(D.depthBias) D.planeVec4 = PLANES_STORED / 4;
    D.compareOp = st->depth_compare_op;
    D.hiz = 1;
    D.minDepthClamp = 0.0f;  // no VK_EXT_depth_range_unrestricted: clamp to [0,1] (PixelProcessor.cpp:106-128)
    D.maxDepthClamp = 1.0f;
    uint32_t opC = simplify_op(st->color_blend_op, st->src_color_factor, st->dst_color_factor);
    uint32_t opA = simplify_op(st->alpha_blend_op, st->src_alpha_factor, st->dst_alpha_factor);
    D.blend = st->blend_enable && (opC != OP_SRC_EXT || opA != OP_SRC_EXT) && st->color_write_mask != 0;
    D.srcC = st->src_color_factor; D.dstC = st->dst_color_factor; D.opC = opC;
    D.srcA = st->src_alpha_factor; D.dstA = st->dst_alpha_factor; D.opA = opA;
    D.blendAlpha = D.srcC == SWGB_BLEND_SRC_ALPHA && D.dstC == SWGB_BLEND_ONE_MINUS_SRC_ALPHA && D.opC == SWGB_BLEND_OP_ADD &&
                   D.srcA == SWGB_BLEND_SRC_ALPHA && D.dstA == SWGB_BLEND_ONE_MINUS_SRC_ALPHA && D.opA == SWGB_BLEND_OP_ADD;
    D.writeMask = st->color_write_mask & 0xFu;
    {
        // B8G8R8A8 stores R in byte 2 and B in byte 0
        const bool bgra = st->color_format == SWGB_FORMAT_B8G8R8A8_UNORM || st->color_format == SWGB_FORMAT_B8G8R8A8_SRGB;
        D.writeBytes = 0;
        for(int c = 0; c < 4; c++)
            if(D.writeMask & (1u << c)) D.writeBytes |= 0xFFu << (8 * (bgra && c != 3 ? 2 - c : c));
    }
    D.ms = (int)st->sample_count;
    D.colorSlice = st->color_slice_bytes;
    D.depthSlice = st->depth_slice_bytes;
    D.cf = (st->color_format == SWGB_FORMAT_R8G8B8A8_UNORM || st->color_format == SWGB_FORMAT_R8G8B8A8_SRGB) ? CF_RGBA8
           : (st->color_format == SWGB_FORMAT_B8G8R8A8_UNORM || st->color_format == SWGB_FORMAT_B8G8R8A8_SRGB) ? CF_BGRA8
           : (st->color_format == SWGB_FORMAT_R16G16B16A16_SFLOAT ? CF_RGBA16F : CF_RGBA32F);
    // sRGB-encoded 8-bit attachment: blend reads decode, writes encode R, G, B
    D.colorSRGB = st->color_format == SWGB_FORMAT_R8G8B8A8_SRGB || st->color_format == SWGB_FORMAT_B8G8R8A8_SRGB;
    D.depth16 = st->depth_format == SWGB_FORMAT_D16_UNORM;
    D.color = (uint8_t *)st->color;
    D.colorPitch = st->color_pitch_bytes;
    D.depth = (uint8_t *)st->depth;
    D.depthPitch = st->depth_pitch_bytes;
    // 16-byte colour rows and 4-pixel depth groups (16 bytes D32F, 8 bytes D16)
    const uint32_t dAlign = D.depth16 ? 8u : 16u;
    D.vec16 = ((uintptr_t)D.color % 16 == 0) && (D.colorPitch % 16 == 0) &&
              (!(D.depthTest || D.depthBounds) || (((uintptr_t)D.depth % dAlign == 0) && (D.depthPitch % dAlign == 0)));

    if(D.fs == SWGB_FS_TEX_X_VCOLOR)
    {
        const swgb_texture &t = st->texture;
        if(t.format == SWGB_FORMAT_R8G8B8A8_UNORM || t.format == SWGB_FORMAT_B8G8R8A8_UNORM || t.format == SWGB_FORMAT_R8G8B8A8_SRGB ||
           t.format == SWGB_FORMAT_B8G8R8A8_SRGB)
        {
            D.texFloat = 0;
            D.texBGRA = t.format == SWGB_FORMAT_B8G8R8A8_UNORM || t.format == SWGB_FORMAT_B8G8R8A8_SRGB;
            D.texSRGB = t.format == SWGB_FORMAT_R8G8B8A8_SRGB || t.format == SWGB_FORMAT_B8G8R8A8_SRGB;
        }
        else if(t.format == SWGB_FORMAT_R16G16B16A16_SFLOAT) D.texFloat = 1;
        else if(t.format == SWGB_FORMAT_R32G32B32A32_SFLOAT) D.texFloat = 2;
        else return set_error(SWGB_UNSUPPORTED_STATE, "texture format");
        if(t.level_count < 1 || t.level_count > SWGB_MAX_MIP_LEVELS) return set_error(SWGB_INVALID_ARG, "texture level_count");
        if(t.mag_filter != t.min_filter) return set_error(SWGB_UNSUPPORTED_STATE, "mixed min/mag filters");
        // REPEAT, MIRRORED_REPEAT, CLAMP_TO_EDGE, CLAMP_TO_BORDER, MIRROR_CLAMP_TO_EDGE
        if(t.address_u > SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE || t.address_v > SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE)
            return set_error(SWGB_UNSUPPORTED_STATE, "address mode");
        // border addressing takes the 32-bit filter path for every format
        // (SamplerCore.cpp:173-176); the border texel is in that path's
        // units: getComponentScale() = 0xFF00 for 8-bit textures, 1 for float
        // ones (replaceBorderTexel, :2290-2355)
        D.border = t.address_u == SWGB_ADDRESS_CLAMP_TO_BORDER || t.address_v == SWGB_ADDRESS_CLAMP_TO_BORDER;
        D.floatPath = D.texFloat != 0 || D.border;
        if(D.border)
        {
            const float sc = D.texFloat ? 1.0f : 65280.0f;
            switch(t.border_color)
            {
            case SWGB_BORDER_COLOR_FLOAT_TRANSPARENT_BLACK:
                for(int k = 0; k < 4; k++) D.borderColor[k] = 0.0f;
                break;
            case SWGB_BORDER_COLOR_FLOAT_OPAQUE_BLACK:
                for(int k = 0; k < 3; k++) D.borderColor[k] = 0.0f;
                D.borderColor[3] = sc;
                break;
            case SWGB_BORDER_COLOR_FLOAT_OPAQUE_WHITE:
                for(int k = 0; k < 4; k++) D.borderColor[k] = sc;
                break;
            case SWGB_BORDER_COLOR_FLOAT_CUSTOM_EXT:
                for(int k = 0; k < 4; k++) D.borderColor[k] = sc * t.custom_border_color[k];
                break;
            default: return set_error(SWGB_UNSUPPORTED_STATE, "border colour (float border colours only)");
            }
        }
        D.levelCount = (int)t.level_count;
        for(uint32_t i = 0; i < t.level_count; i++)
        {
            const swgb_texture_level &l = t.levels[i];
            if(!l.buffer || l.width == 0 || l.height == 0 || l.width > 32768 || l.height > 32768 || l.pitch_texels > 32767)
                return set_error(SWGB_INVALID_ARG, "texture level");
            D.lv[i].buf = (const uint8_t *)l.buffer;
            D.lv[i].w = l.width;
            D.lv[i].h = l.height;
            D.lv[i].pitch = l.pitch_texels;
            D.lv[i].uHalf = (0x8000u / l.width) & 0xFFFFu;  // WriteTextureLevelInfo (VkDescriptorSetLayout.cpp:316-321)
            D.lv[i].vHalf = (0x8000u / l.height) & 0xFFFFu;
        }
        D.texW = (float)t.levels[0].width;
        D.texH = (float)t.levels[0].height;
        auto clampLod = [](float l) { return l < 0.0f ? 0.0f : (l > 13.0f ? 13.0f : l); };  // vk::Sampler ClampLod
        D.minLod = clampLod(t.min_lod);
        D.maxLod = clampLod(t.max_lod);
        if(t.level_count == 1) { D.minLod = 0.0f; D.maxLod = 0.0f; }  // SpirvShaderSampling.cpp:88-99
        D.lodBias = t.mip_lod_bias;
        D.texLinear = t.mag_filter == SWGB_FILTER_LINEAR;
        D.mipLinear = t.mipmap_mode == SWGB_MIPMAP_MODE_LINEAR;
        D.addrU = t.address_u;
        D.addrV = t.address_v;
        D.texRepeatTrilinear = t.format == SWGB_FORMAT_R8G8B8A8_UNORM && !D.floatPath && D.texLinear && D.mipLinear &&
                               D.addrU == SWGB_ADDRESS_REPEAT && D.addrV == SWGB_ADDRESS_REPEAT;
        for(uint32_t i = 0; i < t.level_count && D.texRepeatTrilinear; i++)
            if(t.levels[i].width >= 32768 || t.levels[i].height >= 32768 || t.levels[i].pitch_texels >= 32768) D.texRepeatTrilinear = 0;
    }
    set_bins(D, BIN, BIN);
    D.nchunks = (int)((D.count + CHUNK - 1) / CHUNK);
    D.nsuper = (D.nchunks + SUPER - 1) / SUPER;
    return SWGB_OK;
}

// The raster kernel variants (built in swgb_raster.cu, one object per colour
// format).
const RasterKernel &raster_kernel(int v)
{
    static const std::vector<RasterKernel> table = [] {
        std::vector<RasterKernel> t(NRASTER);
        fill_raster_table<CF_RGBA8>(t.data());
        fill_raster_table<CF_RGBA16F>(t.data());
        fill_raster_table<CF_RGBA32F>(t.data());
        fill_raster_table<CF_BGRA8>(t.data());
        return t;
    }();
    return table[v];
}

// Raster kernel index of a draw: its bin shape, colour format and samples.
// Draws with D16_UNORM depth, depth bias, the depth bounds test, the stencil
// test, an sRGB colour attachment, CLAMP_TO_BORDER addressing or an 8-bit
// texture addressed MIRROR_CLAMP_TO_EDGE run the kernels that carry the full
// per-sample pipeline.
inline bool full_pipeline(const DrawParams &D)
{
    const bool mirrorOnce16 = D.fs == SWGB_FS_TEX_X_VCOLOR && !D.floatPath &&
                              (D.addrU == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE || D.addrV == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE);
    return D.depth16 || D.depthBias || D.depthBounds || D.stencilTest || D.colorSRGB || mirrorOnce16 || D.border;
}
inline int raster_variant(const DrawParams &D) { return raster_index(shape_index(D.binW, D.binH), D.hiz != 0, D.ms, D.cf, full_pipeline(D)); }

// Persistent raster grid of one kernel variant: SMs x resident blocks.
swgb_status raster_grid(int device, int v, bool batch, bool setAttr, int &blocks)
{
    const RasterKernel &k = raster_kernel(v);
    const void *fn = batch ? k.fnBatch : k.fn;
    swgb_status s;
    if(setAttr && (s = cuda_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem),
                                  "raster smem attribute")) != SWGB_OK)
        return s;
    int sms = 0, perSM = 0;
    if((s = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count")) != SWGB_OK) return s;
    if((s = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fn, RASTER_THREADS, k.smem), "raster occupancy")) != SWGB_OK)
        return s;
    blocks = (sms > 0 ? sms : 1) * (perSM > 0 ? perSM : 1);
    return SWGB_OK;
}

// Grids of every variant; without setAttr only of the variants whose shared
// memory needs no opt-in (the allocation-free path's single-sample 16x16
// ones), 0 for the others.
swgb_status raster_grids(int device, bool setAttr, int blocks[NRASTER])
{
    swgb_status s;
    for(int v = 0; v < NRASTER; v++)
    {
        blocks[v] = 0;
        if(!setAttr && raster_kernel(v).smem > 48 * 1024) continue;
        if((s = raster_grid(device, v, false, setAttr, blocks[v])) != SWGB_OK) return s;
    }
    return SWGB_OK;
}

void launch_raster(const DrawParams &D, uint32_t blocks, cudaStream_t st) { raster_kernel(raster_variant(D)).launch(D, blocks, st); }

cudaEvent_t take_event(swgb_ctx *ctx)
{
    cudaEvent_t e = nullptr;
    if(!ctx->evFree->empty())
    {
        e = ctx->evFree->back();
        ctx->evFree->pop_back();
    }
    else
        cudaEventCreate(&e);
    return e;
}

// Launch helper: records a CUDA event pair around the launch when timing is on.
template<typename F>
void timed_launch(swgb_ctx *ctx, int kind, F &&launch, cudaStream_t on = nullptr)
{
    cudaEvent_t a = nullptr, b = nullptr;
    const bool timed = ctx->timing && (ctx->timingKinds >> kind & 1u);
    if(!on) on = ctx->stream;
    if(timed)
    {
        a = take_event(ctx);
        b = take_event(ctx);
        cudaEventRecord(a, on);
    }
    launch();
    ctx->launches++;
    if(timed)
    {
        cudaEventRecord(b, on);
        ctx->evPairs->push_back({kind, {a, b}});
    }
}

constexpr size_t BIN_ORDER_SMEM = 200 * 1024;  // bin grids up to 51200 cells are ordered
constexpr uint32_t BIN_LIST_MIN_TRIANGLES = 4096;    // smaller draws walk their bins in k_raster
constexpr uint32_t BIN_LIST_DEFAULT = 1024;          // candidates per bin list
constexpr size_t BIN_LIST_BYTES = (size_t)256 << 20;  // all of a draw's bin lists

// Grows the context's scratch for draw D and points D at it; with order, also
// the scratch of the heaviest-first bin order (and of its split bins) when it
// applies.
swgb_status prepare_scratch(swgb_ctx *ctx, DrawParams &D, bool order = true)
{
    swgb_status s;
    if((s = ensure(ctx->ptv, ctx->ptvCap, (size_t)D.vertexCount * 4, "ptv")) != SWGB_OK) return s;
    const size_t triSlots = ((size_t)D.count + SETUP_THREADS - 1) / SETUP_THREADS * SETUP_THREADS;
    if((s = ensure(ctx->triBox, ctx->triBoxCap, triSlots, "triangle boxes")) != SWGB_OK) return s;
    if((s = ensure(ctx->triInfo, ctx->triInfoCap, triSlots, "triangle records")) != SWGB_OK) return s;
    if((s = ensure(ctx->planes, ctx->planesCap, triSlots * (PLANES_STORED / 4), "plane equations")) != SWGB_OK) return s;
    // span rows: 24 per triangle covers typical meshes; triangles beyond the
    // capacity fall back to walking their edges in k_raster
    size_t spanNeed = (size_t)D.count * 24 + 4096;
    if(ctx->spanRowsLimit && spanNeed > ctx->spanRowsLimit) spanNeed = ctx->spanRowsLimit;
    if((s = ensure(ctx->spans, ctx->spansCap, spanNeed, "span rows")) != SWGB_OK) return s;
    if((s = ensure(ctx->chunkBox, ctx->chunkCap, triSlots / CHUNK, "chunk boxes")) != SWGB_OK) return s;
    if((s = ensure(ctx->superBox, ctx->superCap, (size_t)D.nsuper, "super-chunk boxes")) != SWGB_OK) return s;
    size_t polyNeed = (size_t)D.count * MAX_POLY;
    if((s = ensure(ctx->poly, ctx->polyCap, polyNeed, "clip polygons")) != SWGB_OK) return s;
    D.ptv = ctx->ptv;
    D.triBox = ctx->triBox;
    D.triInfo = ctx->triInfo;
    D.planes = ctx->planes;
    D.spans = ctx->spans;
    D.spanCount = ctx->spanCount;
    D.spanCapacity = ctx->spanRowsLimit ? (ctx->spansCap < ctx->spanRowsLimit ? ctx->spansCap : ctx->spanRowsLimit) : ctx->spansCap;
    D.chunkBox = ctx->chunkBox;
    D.superBox = ctx->superBox;
    D.poly = ctx->poly;
    D.polyCount = ctx->polyCount;
    D.binQueue = ctx->binQueue;
    D.polyCapacity = (uint32_t)(ctx->polyCap / MAX_POLY);
    D.counters = ctx->counters;
    D.error = ctx->error;
    D.srgbLut = ctx->srgbLut;
    if(!ctx->rasterAttr)
    {
        if((s = raster_grids(ctx->device, true, ctx->rasterBlocks)) != SWGB_OK) return s;
        ctx->rasterAttr = true;
    }
    // Longest-first bin order when the bins outnumber the resident raster
    // warps (with fewer, every bin starts at once) and the bin grid's counts
    // fit k_bin_order's shared memory.
    const size_t nbins = (size_t)D.binsX * D.binsY, cells = (size_t)(D.binsX + 1) * (D.binsY + 1);
    if(D.restart)
    {
        const size_t nb = ((size_t)D.count + RESTART_BLOCK - 1) / RESTART_BLOCK;
        if((s = ensure(ctx->restart, ctx->restartCap, (size_t)D.count + 2 * nb, "restart segments")) != SWGB_OK) return s;
        D.restartLocal = ctx->restart;
        D.restartCarry = ctx->restart + D.count + nb;
    }
    D.binDiff = nullptr;
    D.binFirst = nullptr;
    D.binCost = nullptr;
    D.binOrder = nullptr;
    D.binList = nullptr;
    D.binListCount = nullptr;
    D.binListCap = 0;
    if(order && ctx->binListPerBin && D.count >= ctx->binListMinTris && nbins > 0)
    {
        // per-bin candidate lists, BIN_LIST_BYTES at most in all
        size_t per = ctx->binListPerBin;
        if(nbins * per * sizeof(uint32_t) > BIN_LIST_BYTES) per = (BIN_LIST_BYTES / (nbins * sizeof(uint32_t))) & ~(size_t)31;
        if(per >= 32)
        {
            if((s = ensure(ctx->binList, ctx->binListCap, nbins * per + nbins, "bin lists")) != SWGB_OK) return s;
            D.binList = ctx->binList;
            D.binListCount = ctx->binList + nbins * per;
            D.binListCap = (uint32_t)per;
        }
    }
    if(order && nbins > (size_t)ctx->rasterBlocks[raster_variant(D)] * RASTER_WARPS && cells * sizeof(int) <= BIN_ORDER_SMEM)
    {
        if(!ctx->binOrderAttr)
        {
            if((s = cuda_check(cudaFuncSetAttribute(k_bin_order, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BIN_ORDER_SMEM),
                               "bin order smem attribute")) != SWGB_OK)
                return s;
            ctx->binOrderAttr = true;
        }
        if((s = ensure(ctx->binDiff, ctx->binDiffCap, 2 * cells + nbins, "bin counts")) != SWGB_OK) return s;
        // entries of up to two halves per bin, and their count
        if((s = ensure(ctx->binOrder, ctx->binOrderCap, 2 * nbins + 1, "bin order")) != SWGB_OK) return s;
        D.binDiff = ctx->binDiff;
        D.binFirst = ctx->binDiff + cells;
        // the area estimate needs a second grid in the order kernel's shared memory
        if(2 * cells * sizeof(int) <= BIN_ORDER_SMEM) D.binCost = reinterpret_cast<uint32_t *>(ctx->binDiff + cells + nbins);
        D.binOrder = ctx->binOrder;
        D.rasterWarps = ctx->rasterBlocks[raster_variant(D)] * RASTER_WARPS;
        // half bins: the single-sample variants of the common pixel pipeline
        D.binSplit = D.ms == 1 && !D.hiz && !full_pipeline(D);
    }
    return SWGB_OK;
}

// The context's raster configuration applied to a baked draw (four-sample
// draws keep 16x16 bins).
void apply_config(const swgb_ctx *ctx, DrawParams &D)
{
    if(D.ms == 1 && !full_pipeline(D)) set_bins(D, (int)ctx->rasterConfig.bin_width, (int)ctx->rasterConfig.bin_height);
    D.hiz = (int)ctx->rasterConfig.hiz;
}

swgb_status enqueue(swgb_ctx *ctx, DrawParams &D, cudaEvent_t rasterWait = nullptr)
{
    if(D.count == 0) return SWGB_OK;  // Renderer.cpp:187
    swgb_status s;
    if((s = prepare_scratch(ctx, D)) != SWGB_OK) return s;
    const uint32_t nv = D.vertexCount;
    if(D.restart)
    {
        // primitive restart: segment start of every index position (k_setup reads them)
        const uint32_t nb = (D.count + RESTART_BLOCK - 1) / RESTART_BLOCK;
        uint32_t *blockLast = ctx->restart + D.count;
        timed_launch(ctx, SWGB_KERNEL_SETUP, [&] { k_restart_blocks<<<nb, RESTART_BLOCK, 0, ctx->stream>>>(D, ctx->restart, blockLast); });
        timed_launch(ctx, SWGB_KERNEL_SETUP, [&] { k_restart_carry<<<1, 1024, 0, ctx->stream>>>(blockLast, ctx->restart + D.count + nb, nb); });
    }
    timed_launch(ctx, SWGB_KERNEL_VERTEX, [&] { k_vertex<<<(nv + 255) / 256, 256, 0, ctx->stream>>>(D, nv); });
    const uint32_t setupBlocks = (uint32_t)((D.count + SETUP_THREADS - 1) / SETUP_THREADS);
    timed_launch(ctx, SWGB_KERNEL_SETUP, [&] { k_setup<<<setupBlocks, SETUP_THREADS, 0, ctx->stream>>>(D); });
    // the bin order (one block) and the bin lists depend on the setup stage
    // only: with both, the order runs on the side stream beside the lists
    const bool fork = D.binOrder && D.binList && ctx->side;
    if(fork)
    {
        cudaEventRecord(ctx->sideFork, ctx->stream);
        cudaStreamWaitEvent(ctx->side, ctx->sideFork, 0);
    }
    if(D.binOrder)
    {
        const size_t smem = (size_t)(D.binsX + 1) * (D.binsY + 1) * sizeof(int) * (D.binCost ? 2 : 1);
        cudaStream_t on = fork ? ctx->side : ctx->stream;
        timed_launch(ctx, SWGB_KERNEL_BIN_ORDER, [&] { k_bin_order<<<1, BIN_ORDER_THREADS, smem, on>>>(D); }, on);
    }
    if(D.binList)
    {
        const uint32_t blocks = (uint32_t)((D.binsX * D.binsY + BIN_LIST_WARPS - 1) / BIN_LIST_WARPS);
        timed_launch(ctx, SWGB_KERNEL_BIN_ORDER, [&] { k_bin_list<<<blocks, 32 * BIN_LIST_WARPS, 0, ctx->stream>>>(D); });
    }
    if(fork)
    {
        cudaEventRecord(ctx->sideJoin, ctx->side);
        cudaStreamWaitEvent(ctx->stream, ctx->sideJoin, 0);
    }
    if(D.binsX > 0 && D.binsY > 0)
    {
        uint32_t blocks = (uint32_t)((D.binsX * D.binsY + RASTER_WARPS - 1) / RASTER_WARPS);
        if(blocks > (uint32_t)ctx->rasterBlocks[raster_variant(D)]) blocks = (uint32_t)ctx->rasterBlocks[raster_variant(D)];
        // the textures may still be arriving on another stream
        if(rasterWait) cudaStreamWaitEvent(ctx->stream, rasterWait, 0);
        timed_launch(ctx, SWGB_KERNEL_RASTER, [&] { launch_raster(D, blocks, ctx->stream); });
    }
    return cuda_check(cudaGetLastError(), "kernel launch");
}

}  // namespace

// --------------------------------------------------------------------------
// Batched draws (swgb_draw_batch)
// --------------------------------------------------------------------------

struct BatchState {
    // scratch shared by the draws of one segment
    float4 *ptv = nullptr; size_t ptvCap = 0;
    double *ptv64 = nullptr; size_t ptv64Cap = 0;  // adjoint segments only
    short4 *triBox = nullptr; size_t triBoxCap = 0;
    TriInfo *triInfo = nullptr; size_t triInfoCap = 0;
    float4 *planes = nullptr; size_t planesCap = 0;
    short4 *chunk = nullptr; size_t chunkCap = 0;
    int4 *super = nullptr; size_t superCap = 0;
    uint32_t *spans = nullptr; size_t spansCap = 0;
    int2 *poly = nullptr; size_t polyCap = 0;
    unsigned int *queue = nullptr;
    // descriptors: device copy and pinned staging
    unsigned char *desc = nullptr; size_t descCap = 0;
    unsigned char *stage = nullptr; size_t stageCap = 0;
    cudaEvent_t stageFree = nullptr;
    bool stagePending = false;
    // graph per raster variant, valid for one scratch/descriptor generation
    cudaGraphExec_t graph[NRASTER + 2] = {};  // raster variants, then adjoint 1 / 4 samples
    uint64_t graphGen[NRASTER + 2] = {};
    uint64_t gen = 1;
    cudaStream_t captureStream = nullptr;
    int vertexBlocks = 0, setupBlocks = 0;
    int rasterBlocks[NRASTER] = {};  // persistent grid per raster variant
};

template<typename T>
swgb_status ensure_gen(T *&ptr, size_t &cap, size_t need, BatchState &B, const char *what)
{
    if(need <= cap && ptr) return SWGB_OK;
    size_t grow = need + need / 4 + 1024;
    swgb_status s = ensure(ptr, cap, grow, what);
    if(s == SWGB_OK) B.gen++;
    return s;
}

// Attachment bytes a draw writes, as rectangles in a frame per row pitch:
// address = origin + row * pitch + col, 0 <= col < pitch, origin the lowest
// attachment address of the call.  Colour planes count whole bins within the
// scissor (bins are written back whole); depth planes count when the depth
// test is on.
struct TouchRect {
    uint32_t pitch;
    int64_t row0, row1, col0, col1;
};

inline bool touch_overlap(const TouchRect &a, const TouchRect &b)
{
    return a.pitch == b.pitch && a.row0 < b.row1 && b.row0 < a.row1 && a.col0 < b.col1 && b.col0 < a.col1;
}

void plane_rects(uintptr_t base, uintptr_t origin, uint32_t pitch, int64_t x0b, int64_t x1b, int y0, int y1, std::vector<TouchRect> &out)
{
    if(x1b <= x0b || y1 <= y0 || pitch == 0) return;
    const uintptr_t rel = base - origin;
    int64_t r = (int64_t)(rel / pitch), c = (int64_t)(rel % pitch);
    int64_t sc = c + x0b, ec = c + x1b;
    const int64_t k = sc / pitch;
    r += k;
    sc -= k * pitch;
    ec -= k * pitch;
    if(ec - sc > (int64_t)pitch)  // rows longer than the pitch overlap each other: whole rows
        out.push_back({pitch, r + y0, r + y1 + 1, 0, (int64_t)pitch});
    else if(ec <= (int64_t)pitch)
        out.push_back({pitch, r + y0, r + y1, sc, ec});
    else
    {
        out.push_back({pitch, r + y0, r + y1, sc, (int64_t)pitch});
        out.push_back({pitch, r + y0 + 1, r + y1 + 1, 0, ec - (int64_t)pitch});
    }
}

void draw_writes(const DrawParams &D, uintptr_t origin, std::vector<TouchRect> &out)
{
    out.clear();
    const int cbpp = 4 * color_words(D.cf);
    // bins cover the scissor rounded out to BIN on the left; the write-back
    // clips to the scissor, so the scissor is the written rectangle
    for(int q = 0; q < D.ms; q++)
    {
        plane_rects((uintptr_t)D.color + (uintptr_t)q * D.colorSlice, origin, D.colorPitch, (int64_t)D.sx0 * cbpp,
                    (int64_t)D.sx1 * cbpp, D.sy0, D.sy1, out);
        if(D.stencilTest)  // read by the test, maybe written: either orders the draw
            plane_rects((uintptr_t)D.stencil + (uintptr_t)q * D.stencilSlice, origin, D.stencilPitch, (int64_t)D.sx0, (int64_t)D.sx1,
                        D.sy0, D.sy1, out);
        if(D.depthTest || D.depthBounds)  // written, or read by the bounds test: either orders the draw
            plane_rects((uintptr_t)D.depth + (uintptr_t)q * D.depthSlice, origin, D.depthPitch, (int64_t)D.sx0 * (D.depth16 ? 2 : 4),
                        (int64_t)D.sx1 * (D.depth16 ? 2 : 4), D.sy0, D.sy1, out);
    }
}

// Byte extent [lo, hi) of a rectangle.
inline std::pair<uintptr_t, uintptr_t> rect_extent(const TouchRect &r, uintptr_t origin)
{
    return {origin + (uintptr_t)(r.row0 * r.pitch + r.col0), origin + (uintptr_t)((r.row1 - 1) * r.pitch + r.col1)};
}

// Union of byte intervals, kept merged.
struct IntervalSet {
    std::map<uintptr_t, uintptr_t> iv;
    bool overlaps(uintptr_t lo, uintptr_t hi) const
    {
        if(lo >= hi) return false;
        auto it = iv.upper_bound(lo);
        if(it != iv.begin() && std::prev(it)->second > lo) return true;
        return it != iv.end() && it->first < hi;
    }
    void insert(uintptr_t lo, uintptr_t hi)
    {
        if(lo >= hi) return;
        auto it = iv.upper_bound(lo);
        if(it != iv.begin() && std::prev(it)->second >= lo)
        {
            --it;
            lo = it->first;
            hi = std::max(hi, it->second);
            it = iv.erase(it);
        }
        while(it != iv.end() && it->first <= hi)
        {
            hi = std::max(hi, it->second);
            it = iv.erase(it);
        }
        iv[lo] = hi;
    }
    void clear() { iv.clear(); }
};

// Bytes a draw reads besides its attachments: vertex bindings, index buffer,
// texture levels.
void draw_reads(const swgb_pipeline_state &st, const swgb_draw_args &a, const DrawParams &D,
                std::vector<std::pair<uintptr_t, uintptr_t>> &out)
{
    out.clear();
    // vertices [firstVertex, firstVertex + vertexCount) (non-indexed) or
    // [baseVertex, baseVertex + vertexCount) (indexed), widened to both
    const int64_t first = std::min<int64_t>(0, D.baseVertex);
    const int64_t last = (int64_t)D.firstVertex + std::max<int64_t>(0, D.baseVertex) + D.vertexCount;
    for(int i = 0; i < D.nattr; i++)
    {
        const intptr_t lo = (intptr_t)D.vbuf[i] + (intptr_t)(first * D.vstride[i]);
        const intptr_t hi = (intptr_t)D.vbuf[i] + (intptr_t)(last * D.vstride[i]) + 16;
        out.push_back({(uintptr_t)lo, (uintptr_t)hi});
    }
    if(a.index_type != SWGB_INDEX_TYPE_NONE && a.indices)
    {
        const uintptr_t lo = (uintptr_t)a.indices;
        const uintptr_t isz = a.index_type == SWGB_INDEX_TYPE_UINT16 ? 2 : (a.index_type == SWGB_INDEX_TYPE_UINT8 ? 1 : 4);
        const uintptr_t n = D.topology == SWGB_TOPOLOGY_TRIANGLE_LIST ? (uintptr_t)a.count * 3 : (uintptr_t)a.count + 2;
        out.push_back({lo, lo + n * isz});
    }
    if(D.fs == SWGB_FS_TEX_X_VCOLOR)
    {
        const uintptr_t tb = D.texFloat == 0 ? 4 : D.texFloat == 1 ? 8 : 16;
        for(uint32_t l = 0; l < st.texture.level_count && l < SWGB_MAX_MIP_LEVELS; l++)
        {
            const swgb_texture_level &lv = st.texture.levels[l];
            const uintptr_t lo = (uintptr_t)lv.buffer;
            out.push_back({lo, lo + (uintptr_t)lv.pitch_texels * lv.height * tb});
        }
    }
}

// Splits draws into consecutive segments that each run as one batch: same
// raster variant, no two draws of a segment write overlapping attachment
// bytes, and no draw reads bytes another draw of its segment writes.  Running
// a segment's draws concurrently then gives the sequential result.
void segment_batch(const std::vector<DrawParams> &D, const std::vector<uint32_t> &src, const swgb_pipeline_state *states,
                   const swgb_draw_args *args, std::vector<std::pair<uint32_t, uint32_t>> &segs)
{
    uintptr_t origin = UINTPTR_MAX;
    for(const DrawParams &d : D)
    {
        origin = std::min(origin, (uintptr_t)d.color);
        if(d.depthTest) origin = std::min(origin, (uintptr_t)d.depth);
    }
    std::unordered_map<uint64_t, std::vector<TouchRect>> cells;  // write rects by (pitch, 64-row, 4 KiB-column) cell
    std::map<uint32_t, IntervalSet> writesByPitch;
    IntervalSet reads;
    std::vector<TouchRect> w;
    std::vector<std::pair<uintptr_t, uintptr_t>> r;
    std::vector<uint64_t> keys;
    auto cellKeys = [&keys](const TouchRect &t) {
        keys.clear();
        for(int64_t y = t.row0 >> 6; y <= (t.row1 - 1) >> 6; y++)
            for(int64_t x = t.col0 >> 12; x <= (t.col1 - 1) >> 12; x++)
                keys.push_back(((uint64_t)t.pitch << 40) ^ ((uint64_t)(y & 0xFFFFF) << 20) ^ (uint64_t)(x & 0xFFFFF));
    };
    uint32_t start = 0;
    for(uint32_t i = 0; i < (uint32_t)D.size(); i++)
    {
        draw_writes(D[i], origin, w);
        draw_reads(states[src[i]], args[src[i]], D[i], r);
        bool conflict = i > start && raster_variant(D[i]) != raster_variant(D[start]);
        for(size_t k = 0; k < w.size() && !conflict; k++)
        {
            const TouchRect &t = w[k];
            cellKeys(t);
            for(uint64_t key : keys)
            {
                auto it = cells.find(key);
                if(it == cells.end()) continue;
                for(const TouchRect &o : it->second)
                    if(touch_overlap(t, o)) { conflict = true; break; }
                if(conflict) break;
            }
            const auto ext = rect_extent(t, origin);
            if(!conflict && reads.overlaps(ext.first, ext.second)) conflict = true;
            for(auto &wp : writesByPitch)
                if(!conflict && wp.first != t.pitch && wp.second.overlaps(ext.first, ext.second)) conflict = true;
        }
        for(size_t k = 0; k < r.size() && !conflict; k++)
            for(auto &wp : writesByPitch)
                if(wp.second.overlaps(r[k].first, r[k].second)) { conflict = true; break; }
        if(conflict)
        {
            segs.push_back({start, i});
            start = i;
            cells.clear();
            writesByPitch.clear();
            reads.clear();
        }
        for(const TouchRect &t : w)
        {
            cellKeys(t);
            for(uint64_t key : keys) cells[key].push_back(t);
            const auto ext = rect_extent(t, origin);
            writesByPitch[t.pitch].insert(ext.first, ext.second);
        }
        for(auto &e : r) reads.insert(e.first, e.second);
    }
    if(start < (uint32_t)D.size()) segs.push_back({start, (uint32_t)D.size()});
}

void launch_raster_batch(int variant, const BatchPtrs &P, uint32_t blocks, cudaStream_t st)
{
    raster_kernel(variant).launchBatch(P, blocks, st);
}

swgb_status batch_init(swgb_ctx *ctx)
{
    if(ctx->batch) return SWGB_OK;
    BatchState *B = new BatchState();
    swgb_status s;
    int sms = 1, perSM = 1;
    if((s = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "SM count")) != SWGB_OK ||
       (s = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_setup_batch, SETUP_THREADS, 0), "setup occupancy")) != SWGB_OK)
    {
        delete B;
        return s;
    }
    for(int v = 0; v < NRASTER; v++)
        if((s = raster_grid(ctx->device, v, true, true, B->rasterBlocks[v])) != SWGB_OK)
        {
            delete B;
            return s;
        }
    B->setupBlocks = std::max(1, sms * std::max(1, perSM));
    B->vertexBlocks = std::max(1, sms * 8);
    if((s = cuda_check(cudaMalloc((void **)&B->queue, sizeof(unsigned int)), "batch queue")) != SWGB_OK ||
       (s = cuda_check(cudaEventCreateWithFlags(&B->stageFree, cudaEventDisableTiming), "batch event")) != SWGB_OK ||
       (s = cuda_check(cudaStreamCreateWithFlags(&B->captureStream, cudaStreamNonBlocking), "capture stream")) != SWGB_OK)
    {
        delete B;
        return s;
    }
    ctx->batch = B;
    return SWGB_OK;
}

void batch_free(BatchState *B)
{
    if(!B) return;
    cudaFree(B->ptv); cudaFree(B->ptv64); cudaFree(B->triBox); cudaFree(B->triInfo); cudaFree(B->planes); cudaFree(B->chunk); cudaFree(B->super);
    cudaFree(B->spans); cudaFree(B->poly); cudaFree(B->queue); cudaFree(B->desc);
    if(B->stage) cudaFreeHost(B->stage);
    if(B->stageFree) cudaEventDestroy(B->stageFree);
    for(int v = 0; v < NRASTER + 2; v++)
        if(B->graph[v]) cudaGraphExecDestroy(B->graph[v]);
    if(B->captureStream) cudaStreamDestroy(B->captureStream);
    delete B;
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Descriptor image of a segment of n draws: header | draws | vStart | sStart
// | bStart | (adjoint batches) AdjParams.  Returns its size in bytes.
struct DescLayout {
    size_t offDraws, offV, offS, offB, offAdj, bytes;
};

DescLayout desc_layout(uint32_t n, bool adjoint)
{
    DescLayout L;
    L.offDraws = align_up(sizeof(BatchHeader), 64);
    L.offV = align_up(L.offDraws + (size_t)n * sizeof(DrawParams), 64);
    L.offS = align_up(L.offV + (size_t)(n + 1) * 4, 64);
    L.offB = align_up(L.offS + (size_t)(n + 1) * 4, 64);
    L.offAdj = align_up(L.offB + (size_t)(n + 1) * 4, 64);
    L.bytes = align_up(L.offAdj + (adjoint ? (size_t)n * sizeof(AdjParams) : 0), 256);
    return L;
}

void launch_adjoint_batch(int ms4, const BatchPtrs &P, uint32_t blocks, cudaStream_t st, uint8_t *scratch)
{
    if(ms4) k_adjoint_batch<4><<<blocks, ADJ_THREADS, ADJ_WARPS * sizeof(AdjShared<4>), st>>>(P, scratch);
    else k_adjoint_batch<1><<<blocks, ADJ_THREADS, ADJ_WARPS * sizeof(AdjShared<1>), st>>>(P, scratch);
}

// Enqueues one segment: descriptors (staged at stageOff), then the batched
// vertex and setup kernels and the raster kernel (or, with adj, the adjoint
// kernel), as a graph replay unless kernel timing is on.
swgb_status enqueue_segment(swgb_ctx *ctx, std::vector<DrawParams> &draws, uint32_t first, uint32_t last, size_t &stageOff,
                            const AdjParams *adj = nullptr)
{
    BatchState &B = *ctx->batch;
    const uint32_t n = last - first;
    std::vector<uint32_t> vStart(n + 1), sStart(n + 1), bStart(n + 1);
    uint64_t verts = 0, vblocks = 0, sblocks = 0, bins = 0, nsuper = 0;
    for(uint32_t k = 0; k < n; k++)
    {
        const DrawParams &d = draws[first + k];
        vStart[k] = (uint32_t)vblocks;
        sStart[k] = (uint32_t)sblocks;
        bStart[k] = (uint32_t)bins;
        const uint32_t vc = d.count ? d.vertexCount : 0;
        vblocks += (vc + 255) / 256;
        verts += (uint64_t)((vc + 255) / 256) * 256;
        sblocks += (d.count + SETUP_THREADS - 1) / SETUP_THREADS;
        bins += d.count ? (uint64_t)d.binsX * d.binsY : 0;
        nsuper += (uint64_t)d.nsuper;
    }
    vStart[n] = (uint32_t)vblocks;
    sStart[n] = (uint32_t)sblocks;
    bStart[n] = (uint32_t)bins;
    if(vblocks > 0xFFFFFFFFull || sblocks > 0xFFFFFFFFull || bins > 0xFFFFFFFFull || (uint64_t)n * sizeof(DrawParams) > 0xF0000000ull)
        return set_error(SWGB_UNSUPPORTED_STATE, "batch too large");
    swgb_status s;
    const uint64_t triSlots = sblocks * SETUP_THREADS;
    if((s = ensure_gen(B.ptv, B.ptvCap, (size_t)verts * 4, B, "batch ptv")) != SWGB_OK) return s;
    if(adj && (s = ensure_gen(B.ptv64, B.ptv64Cap, (size_t)verts * 6, B, "batch fp64 clip coordinates")) != SWGB_OK) return s;
    if((s = ensure_gen(B.triBox, B.triBoxCap, (size_t)triSlots, B, "batch boxes")) != SWGB_OK) return s;
    if((s = ensure_gen(B.triInfo, B.triInfoCap, (size_t)triSlots, B, "batch records")) != SWGB_OK) return s;
    if((s = ensure_gen(B.planes, B.planesCap, (size_t)triSlots * (PLANES_STORED / 4), B, "batch plane equations")) != SWGB_OK) return s;
    if((s = ensure_gen(B.chunk, B.chunkCap, (size_t)triSlots / CHUNK, B, "batch chunks")) != SWGB_OK) return s;
    if((s = ensure_gen(B.super, B.superCap, (size_t)nsuper + 1, B, "batch super boxes")) != SWGB_OK) return s;
    uint64_t tris = 0;
    for(uint32_t k = 0; k < n; k++) tris += draws[first + k].count;
    if((s = ensure_gen(B.spans, B.spansCap, (size_t)(tris * 24 + 4096), B, "batch spans")) != SWGB_OK) return s;
    if((s = ensure_gen(B.poly, B.polyCap, (size_t)(tris + 1) * MAX_POLY, B, "batch polygons")) != SWGB_OK) return s;
    // per-draw scratch windows
    uint64_t vOff = 0, sOff = 0, supOff = 0;
    for(uint32_t k = 0; k < n; k++)
    {
        DrawParams &d = draws[first + k];
        d.ptv = B.ptv + vOff * 4;
        d.ptv64 = adj ? B.ptv64 + vOff * 6 : nullptr;
        d.triBox = B.triBox + sOff;
        d.triInfo = B.triInfo + sOff;
        d.planes = B.planes + (size_t)sOff * (PLANES_STORED / 4);
        d.chunkBox = B.chunk + sOff / CHUNK;
        d.superBox = B.super + supOff;
        d.spans = B.spans;
        d.spanCount = ctx->spanCount;
        d.spanCapacity = ctx->spanRowsLimit ? std::min<uint64_t>(B.spansCap, ctx->spanRowsLimit) : B.spansCap;
        d.poly = B.poly;
        d.polyCount = ctx->polyCount;
        d.polyCapacity = (uint32_t)std::min<size_t>(B.polyCap / MAX_POLY, 0xFFFFFFFFu);
        d.counters = ctx->counters;
        d.srgbLut = ctx->srgbLut;
        d.error = ctx->error;
        d.binQueue = B.queue;
        const uint32_t vc = d.count ? d.vertexCount : 0;
        vOff += (uint64_t)((vc + 255) / 256) * 256;
        sOff += (uint64_t)((d.count + SETUP_THREADS - 1) / SETUP_THREADS) * SETUP_THREADS;
        supOff += (uint64_t)d.nsuper;
    }
    const DescLayout L = desc_layout(n, adj != nullptr);
    const size_t bytes = L.bytes;
    if((s = ensure_gen(B.desc, B.descCap, bytes, B, "batch descriptors")) != SWGB_OK) return s;
    unsigned char *img = B.stage + stageOff;
    BatchHeader h = {};
    h.n = n;
    h.vblocks = (uint32_t)vblocks;
    h.sblocks = (uint32_t)sblocks;
    h.bins = (uint32_t)bins;
    h.nsuper = (uint32_t)nsuper;
    h.offDraws = (uint32_t)L.offDraws;
    h.offV = (uint32_t)L.offV;
    h.offS = (uint32_t)L.offS;
    h.offB = (uint32_t)L.offB;
    h.offAdj = (uint32_t)L.offAdj;
    // adjoint over few bins: four warps per bin (quarters)
    h.split = adj && bins < 2ull * (uint64_t)ctx->adjBlocks[draws[first].ms > 1 ? 1 : 0] * ADJ_WARPS ? 4 : 1;
    memcpy(img, &h, sizeof(h));
    memcpy(img + L.offDraws, draws.data() + first, (size_t)n * sizeof(DrawParams));
    memcpy(img + L.offV, vStart.data(), (size_t)(n + 1) * 4);
    memcpy(img + L.offS, sStart.data(), (size_t)(n + 1) * 4);
    memcpy(img + L.offB, bStart.data(), (size_t)(n + 1) * 4);
    if(adj) memcpy(img + L.offAdj, adj + first, (size_t)n * sizeof(AdjParams));
    if((s = cuda_check(cudaMemcpyAsync(B.desc, img, bytes, cudaMemcpyHostToDevice, ctx->stream), "batch descriptors upload")) != SWGB_OK)
        return s;
    stageOff += bytes;

    BatchPtrs P;
    P.hdr = (const BatchHeader *)B.desc;
    P.superAll = B.super;
    P.binQueue = B.queue;
    P.polyCount = ctx->polyCount;
    P.spanCount = ctx->spanCount;
    P.counters = ctx->counters;
    // graph slot: raster variants, then adjoint NRASTER (1 sample) and NRASTER + 1 (4 samples)
    const int variant = adj ? NRASTER + (draws[first].ms > 1 ? 1 : 0) : raster_variant(draws[first]);
    const uint32_t rblocks = (uint32_t)(adj ? ctx->adjBlocks[variant - NRASTER] : B.rasterBlocks[variant]);
    auto third = [&](cudaStream_t st) {
        if(adj) launch_adjoint_batch(variant - NRASTER, P, rblocks, st, ctx->adjScratch);
        else launch_raster_batch(variant, P, rblocks, st);
    };
    if(ctx->timing)
    {
        timed_launch(ctx, SWGB_KERNEL_VERTEX, [&] { k_vertex_batch<<<B.vertexBlocks, 256, 0, ctx->stream>>>(P); });
        timed_launch(ctx, SWGB_KERNEL_SETUP, [&] { k_setup_batch<<<B.setupBlocks, SETUP_THREADS, 0, ctx->stream>>>(P); });
        timed_launch(ctx, adj ? SWGB_KERNEL_ADJOINT : SWGB_KERNEL_RASTER, [&] { third(ctx->stream); });
        return cuda_check(cudaGetLastError(), "batch launch");
    }
    // The graph's kernel parameters point at fixed scratch and descriptor
    // addresses; it is captured again only when one of them moved.
    if(!B.graph[variant] || B.graphGen[variant] != B.gen)
    {
        if(B.graph[variant]) cudaGraphExecDestroy(B.graph[variant]);
        B.graph[variant] = nullptr;
        cudaGraph_t g = nullptr;
        if((s = cuda_check(cudaStreamBeginCapture(B.captureStream, cudaStreamCaptureModeThreadLocal), "begin capture")) != SWGB_OK) return s;
        k_vertex_batch<<<B.vertexBlocks, 256, 0, B.captureStream>>>(P);
        k_setup_batch<<<B.setupBlocks, SETUP_THREADS, 0, B.captureStream>>>(P);
        third(B.captureStream);
        if((s = cuda_check(cudaStreamEndCapture(B.captureStream, &g), "end capture")) != SWGB_OK) return s;
        s = cuda_check(cudaGraphInstantiate(&B.graph[variant], g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        if(s != SWGB_OK) return s;
        B.graphGen[variant] = B.gen;
    }
    timed_launch(ctx, SWGB_KERNEL_BATCH, [&] { cudaGraphLaunch(B.graph[variant], ctx->stream); });
    ctx->launches += 2;  // the graph holds three kernel launches
    return cuda_check(cudaGetLastError(), "graph launch");
}

// Stages the descriptors of every segment of one call (after the previous
// call's uploads have read theirs) and enqueues the segments in order.
swgb_status run_segments(swgb_ctx *ctx, std::vector<DrawParams> &draws, const std::vector<std::pair<uint32_t, uint32_t>> &segs,
                         const AdjParams *adj)
{
    swgb_status s;
    BatchState &B = *ctx->batch;
    size_t need = 0;
    for(auto &sg : segs) need += desc_layout(sg.second - sg.first, adj != nullptr).bytes;
    if(B.stagePending)
    {
        if((s = cuda_check(cudaEventSynchronize(B.stageFree), "staging reuse")) != SWGB_OK) return s;
        B.stagePending = false;
    }
    if(need > B.stageCap)
    {
        if(B.stage) cudaFreeHost(B.stage);
        B.stage = nullptr;
        B.stageCap = 0;
        if((s = cuda_check(cudaMallocHost((void **)&B.stage, need + need / 4), "batch staging")) != SWGB_OK) return s;
        B.stageCap = need + need / 4;
    }
    size_t stageOff = 0;
    for(auto &sg : segs)
        if((s = enqueue_segment(ctx, draws, sg.first, sg.second, stageOff, adj)) != SWGB_OK) return s;
    if((s = cuda_check(cudaEventRecord(B.stageFree, ctx->stream), "staging event")) != SWGB_OK) return s;
    B.stagePending = true;
    return SWGB_OK;
}

swgb_status draw_batch(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n)
{
    std::vector<DrawParams> draws;
    std::vector<uint32_t> src;
    draws.reserve(n);
    for(uint32_t i = 0; i < n; i++)
    {
        if(args[i].count == 0 && !args[i].restart_index_count) continue;  // Renderer.cpp:187
        DrawParams D;
        swgb_status s = bake(&states[i], &args[i], D);
        if(s != SWGB_OK) return s;
        if(D.restart) return set_error(SWGB_UNSUPPORTED_STATE, "swgb_draw_batch: primitive restart needs swgb_draw");
        apply_config(ctx, D);
        draws.push_back(D);
        src.push_back(i);
    }
    if(draws.empty()) return SWGB_OK;
    swgb_status s;
    if((s = batch_init(ctx)) != SWGB_OK) return s;
    std::vector<std::pair<uint32_t, uint32_t>> segs;
    segment_batch(draws, src, states, args, segs);
    // Longest first inside a segment: its draws touch disjoint attachment
    // bytes, so their order changes no result, and the persistent raster warps
    // take the bins of the costliest draws (triangles x bins) first.
    for(const auto &sg : segs)
        std::stable_sort(draws.begin() + sg.first, draws.begin() + sg.second, [](const DrawParams &a, const DrawParams &b) {
            return (uint64_t)a.count * (uint64_t)(a.binsX * a.binsY) > (uint64_t)b.count * (uint64_t)(b.binsX * b.binsY);
        });
    return run_segments(ctx, draws, segs, nullptr);
}

// --------------------------------------------------------------------------
// Adjoint draws (swgb_draw_adjoint, swgb_draw_adjoint_batch)
// --------------------------------------------------------------------------

inline bool aligned(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

// Validates the adjoint's scope and bakes its parameters.
swgb_status bake_adjoint(const swgb_pipeline_state *st, const swgb_draw_args *a, const swgb_adjoint_args *g, const DrawParams &D,
                         AdjParams &A)
{
    if(!g) return set_error(SWGB_INVALID_ARG, "null adjoint arguments");
    if(cf_unorm8(D.cf)) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint needs a float colour attachment");
    if(D.restart) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint: primitive restart is not supported");
    if(D.depth16) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint needs a D32_SFLOAT depth attachment");
    if(D.depthBounds) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint: depth bounds test is not supported");
    if(D.stencilTest) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint: stencil test is not supported");
    if(D.depthBias) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint: depth bias is not supported");
    if(D.fs == SWGB_FS_TEX_X_VCOLOR && !D.texFloat) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint needs a float texture");
    if(D.fs == SWGB_FS_TEX_X_VCOLOR && (D.addrU == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE || D.addrV == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE ||
                                        D.border))
        return set_error(SWGB_UNSUPPORTED_STATE, "adjoint: MIRROR_CLAMP_TO_EDGE / CLAMP_TO_BORDER addressing is not supported");
    if(D.writeMask != 0xFu) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint needs color_write_mask 0xF");
    if(a->count > ADJ_TRI_MASK) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint: too many triangles");
    int over = 0;
    if(st->blend_enable)
    {
        over = st->src_color_factor == SWGB_BLEND_ONE && st->dst_color_factor == SWGB_BLEND_ONE_MINUS_SRC_ALPHA &&
               st->color_blend_op == SWGB_BLEND_OP_ADD && st->src_alpha_factor == SWGB_BLEND_ONE &&
               st->dst_alpha_factor == SWGB_BLEND_ONE_MINUS_SRC_ALPHA && st->alpha_blend_op == SWGB_BLEND_OP_ADD;
        if(!over) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint blends: none or premultiplied OVER only");
    }
    if(!g->grad_color || !aligned(g->grad_color, 16) || g->grad_color_pitch_bytes % 16 || g->grad_color_slice_bytes % 16 ||
       g->grad_color_pitch_bytes < 16u * st->framebuffer_width ||
       (D.ms > 1 && g->grad_color_slice_bytes < (uint64_t)g->grad_color_pitch_bytes * st->framebuffer_height))
        return set_error(SWGB_INVALID_ARG, "grad_color: null, not 16-byte aligned, or pitch/slice too small");
    memset(&A, 0, sizeof(A));
    A.gradColor = (const uint8_t *)g->grad_color;
    A.gradPitch = g->grad_color_pitch_bytes;
    A.rxs = 256.0 / (double)D.WxF;
    A.rx0 = -(double)D.X0xF / (double)D.WxF;
    A.rys = 256.0 / (double)D.HxF;
    A.ry0 = -(double)D.Y0xF / (double)D.HxF;
    A.gradSlice = g->grad_color_slice_bytes;
    for(int c = 0; c < 4; c++) A.clear[c] = g->clear_color[c];
    A.clearDepth = g->clear_depth;
    A.blendOver = over;
    if(D.fs == SWGB_FS_TEX_X_VCOLOR)
        for(int l = 0; l < D.levelCount; l++)
        {
            if(g->grad_texels[l] && !aligned(g->grad_texels[l], 16))
                return set_error(SWGB_INVALID_ARG, "grad_texels: not 16-byte aligned");
            A.gradTex[l] = g->grad_texels[l];
        }
    for(uint32_t i = 0; i < st->attrib_count && i < SWGB_MAX_ATTRIBS; i++)
    {
        const swgb_vertex_attrib &at = st->attribs[i];
        uint8_t *base = (uint8_t *)g->grad_vertices[at.binding];
        if(!base) continue;
        if(!aligned(base, 4) || at.offset % 4 || st->bindings[at.binding].stride % 4)
            return set_error(SWGB_INVALID_ARG, "grad_vertices: not 4-byte aligned");
        A.gradAttr[i] = base + at.offset;
        A.gradStride[i] = st->bindings[at.binding].stride;
    }
    return SWGB_OK;
}

template<int MS>
swgb_status adjoint_grid(int device, int &blocks)
{
    constexpr size_t smem = ADJ_WARPS * sizeof(AdjShared<MS>);
    swgb_status s;
    if((s = cuda_check(cudaFuncSetAttribute(k_adjoint<MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "adjoint smem")) != SWGB_OK ||
       (s = cuda_check(cudaFuncSetAttribute(k_adjoint_batch<MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "adjoint smem")) != SWGB_OK)
        return s;
    int sms = 0, perSM = 0, perSM1 = 0;
    if((s = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count")) != SWGB_OK) return s;
    if((s = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_adjoint_batch<MS>, ADJ_THREADS, smem), "adjoint occupancy")) != SWGB_OK ||
       (s = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM1, k_adjoint<MS>, ADJ_THREADS, smem), "adjoint occupancy")) != SWGB_OK)
        return s;
    perSM = std::min(perSM, perSM1);
    blocks = (sms > 0 ? sms : 1) * (perSM > 0 ? perSM : 1);
    return SWGB_OK;
}

swgb_status adjoint_init(swgb_ctx *ctx)
{
    if(ctx->adjAttr) return SWGB_OK;
    swgb_status s;
    if((s = adjoint_grid<1>(ctx->device, ctx->adjBlocks[0])) != SWGB_OK || (s = adjoint_grid<4>(ctx->device, ctx->adjBlocks[1])) != SWGB_OK)
        return s;
    const size_t warps = (size_t)std::max(ctx->adjBlocks[0], ctx->adjBlocks[1]) * ADJ_WARPS;
    if((s = cuda_check(cudaMalloc((void **)&ctx->adjScratch, warps * ADJ_REGION_BYTES), "adjoint scratch")) != SWGB_OK) return s;
    ctx->adjAttr = true;
    return SWGB_OK;
}

swgb_status draw_adjoint(swgb_ctx *ctx, const swgb_pipeline_state *st, const swgb_draw_args *a, const swgb_adjoint_args *g)
{
    DrawParams D;
    swgb_status s = bake(st, a, D);
    if(s != SWGB_OK) return s;
    AdjParams A;
    if((s = bake_adjoint(st, a, g, D, A)) != SWGB_OK) return s;
    if(D.count == 0) return SWGB_OK;
    if((s = adjoint_init(ctx)) != SWGB_OK) return s;
    if((s = prepare_scratch(ctx, D, false)) != SWGB_OK) return s;
    if((s = ensure(ctx->ptv64, ctx->ptv64Cap, (size_t)D.vertexCount * 6, "fp64 clip coordinates")) != SWGB_OK) return s;
    D.ptv64 = ctx->ptv64;
    const uint32_t nv = D.vertexCount;
    timed_launch(ctx, SWGB_KERNEL_VERTEX, [&] { k_vertex<<<(nv + 255) / 256, 256, 0, ctx->stream>>>(D, nv); });
    const uint32_t setupBlocks = (uint32_t)((D.count + SETUP_THREADS - 1) / SETUP_THREADS);
    timed_launch(ctx, SWGB_KERNEL_SETUP, [&] { k_setup<<<setupBlocks, SETUP_THREADS, 0, ctx->stream>>>(D); });
    if(D.binsX > 0 && D.binsY > 0)
    {
        const int v = D.ms > 1 ? 1 : 0;
        const uint32_t bins = (uint32_t)(D.binsX * D.binsY);
        const int split = bins < 2u * (uint32_t)ctx->adjBlocks[v] * ADJ_WARPS ? 4 : 1;  // few bins: quarter them
        uint32_t blocks = (bins * split + ADJ_WARPS - 1) / ADJ_WARPS;
        if(blocks > (uint32_t)ctx->adjBlocks[v]) blocks = (uint32_t)ctx->adjBlocks[v];
        timed_launch(ctx, SWGB_KERNEL_ADJOINT, [&] {
            if(v) k_adjoint<4><<<blocks, ADJ_THREADS, ADJ_WARPS * sizeof(AdjShared<4>), ctx->stream>>>(D, A, ctx->adjScratch, split);
            else k_adjoint<1><<<blocks, ADJ_THREADS, ADJ_WARPS * sizeof(AdjShared<1>), ctx->stream>>>(D, A, ctx->adjScratch, split);
        });
    }
    return cuda_check(cudaGetLastError(), "adjoint launch");
}

swgb_status draw_adjoint_batch(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args,
                               const swgb_adjoint_args *adjs, uint32_t n)
{
    std::vector<DrawParams> draws;
    std::vector<AdjParams> adj;
    draws.reserve(n);
    adj.reserve(n);
    for(uint32_t i = 0; i < n; i++)
    {
        DrawParams D;
        swgb_status s = bake(&states[i], &args[i], D);
        if(s != SWGB_OK) return s;
        AdjParams A;
        if((s = bake_adjoint(&states[i], &args[i], &adjs[i], D, A)) != SWGB_OK) return s;
        if(args[i].count == 0) continue;
        draws.push_back(D);
        adj.push_back(A);
    }
    if(draws.empty()) return SWGB_OK;
    swgb_status s;
    if((s = batch_init(ctx)) != SWGB_OK || (s = adjoint_init(ctx)) != SWGB_OK) return s;
    // adjoints only read attachments and add to gradients, so draws never
    // conflict; segments split by sample count only
    std::vector<std::pair<uint32_t, uint32_t>> segs;
    uint32_t start = 0;
    for(uint32_t i = 1; i <= (uint32_t)draws.size(); i++)
        if(i == (uint32_t)draws.size() || (draws[i].ms > 1) != (draws[start].ms > 1))
        {
            segs.push_back({start, i});
            start = i;
        }
    return run_segments(ctx, draws, segs, adj.data());
}

// --------------------------------------------------------------------------
// Allocation-free draws (swgb_draw_noalloc)
//
// Some callers cannot allocate device memory at draw time: a driver-style
// caller running inside a CUDA stream capture (graph capture forbids
// cudaMalloc), a caller whose memory pool is owned by another allocator, or a
// real-time loop that must not touch the allocator.  For them the draw's
// scratch lives in one file-scope __device__ array of fixed size, which every
// GPU that loads this library holds until the process exits.
// --------------------------------------------------------------------------

constexpr size_t NA_ALIGN = 256;
constexpr size_t na_up(size_t x) { return (x + NA_ALIGN - 1) / NA_ALIGN * NA_ALIGN; }
constexpr uint32_t NA_TRIS = SWGB_NOALLOC_MAX_TRIANGLES;
constexpr uint32_t NA_VERTS = SWGB_NOALLOC_MAX_VERTICES;
constexpr uint32_t NA_SLOTS = (NA_TRIS + SETUP_THREADS - 1) / SETUP_THREADS * SETUP_THREADS;
constexpr uint32_t NA_CHUNKS = NA_SLOTS / CHUNK;
constexpr uint32_t NA_SUPER = (NA_CHUNKS + SUPER - 1) / SUPER;
constexpr uint64_t NA_SPAN_ROWS = (uint64_t)NA_TRIS * 24;
constexpr size_t NA_OFF_PTV = 0;
constexpr size_t NA_OFF_BOX = na_up(NA_OFF_PTV + (size_t)NA_VERTS * 4 * sizeof(float4));
constexpr size_t NA_OFF_INFO = na_up(NA_OFF_BOX + (size_t)NA_SLOTS * sizeof(short4));
constexpr size_t NA_OFF_PLANES = na_up(NA_OFF_INFO + (size_t)NA_SLOTS * sizeof(TriInfo));
constexpr size_t NA_OFF_CHUNK = na_up(NA_OFF_PLANES + (size_t)NA_SLOTS * PLANES_STORED * sizeof(float));
constexpr size_t NA_OFF_SUPER = na_up(NA_OFF_CHUNK + (size_t)NA_CHUNKS * sizeof(short4));
constexpr size_t NA_OFF_SPANS = na_up(NA_OFF_SUPER + (size_t)NA_SUPER * sizeof(int4));
constexpr size_t NA_OFF_POLY = na_up(NA_OFF_SPANS + (size_t)NA_SPAN_ROWS * sizeof(uint32_t));
constexpr size_t NA_OFF_WORDS = na_up(NA_OFF_POLY + (size_t)NA_TRIS * MAX_POLY * sizeof(int2));
// words: counters[8] (u64), spanCount (u64), polyCount (u32), binQueue (u32), error (i32)
constexpr size_t NA_WORDS_BYTES = 8 * 8 + 8 + 4 + 4 + 4;
constexpr size_t NA_BYTES = na_up(NA_OFF_WORDS + NA_WORDS_BYTES);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

struct NoAllocDevice {
    bool ready;
    unsigned char *base;  // device address of g_noalloc_scratch on this device
    int rasterBlocks[NRASTER];
};
static NoAllocDevice g_noalloc_dev[64];
static std::mutex g_noalloc_mu;

// Once per device, with that device current: resolve the device address of
// the scratch array (the host-side symbol is only a stand-in and must never
// reach a kernel) and size the persistent raster grid.
swgb_status noalloc_device(int dev, NoAllocDevice *&out)
{
    if(dev < 0 || dev >= 64) return set_error(SWGB_INVALID_ARG, "device index beyond 63");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if(!d.ready)
    {
        void *ptr = nullptr;
        swgb_status s = cuda_check(cudaGetSymbolAddress(&ptr, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
        if(s != SWGB_OK) return s;
        // set-up, once per device: the raster kernels' shared-memory opt-in
        // (a function attribute, no allocation) and their grids
        if((s = raster_grids(dev, true, d.rasterBlocks)) != SWGB_OK) return s;
        d.base = (unsigned char *)ptr;
        d.ready = true;
    }
    out = &d;
    return SWGB_OK;
}

extern "C" {

int swgb_abi_version(void) { return SWGB_ABI_VERSION; }

const char *swgb_last_error(void) { return g_error.c_str(); }

swgb_status swgb_ctx_create(int device, void *stream, swgb_ctx **out)
{
    if(!out) return set_error(SWGB_INVALID_ARG, "out is null");
    *out = nullptr;
    int n = 0;
    if(cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return set_error(SWGB_NO_DEVICE, "no CUDA device");
    if(device < 0 || device >= n) return set_error(SWGB_INVALID_ARG, "device index");
    swgb_status s = cuda_check(cudaSetDevice(device), "cudaSetDevice");
    if(s != SWGB_OK) return s;
    swgb_ctx *c = new swgb_ctx();
    memset(c, 0, sizeof(*c));
    c->device = device;
    c->rasterConfig = {BIN, BIN, 1u, 0u};
    c->evFree = new std::vector<cudaEvent_t>();
    c->evPairs = new std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>>();
    if(stream)
        c->stream = (cudaStream_t)stream;
    else
    {
        if((s = cuda_check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream")) != SWGB_OK) { delete c; return s; }
        c->ownStream = true;
    }
    if(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&c->sideFork, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&c->sideJoin, cudaEventDisableTiming) != cudaSuccess)
    {
        // without them the bin order runs on the context's stream
        cudaGetLastError();
        if(c->side) cudaStreamDestroy(c->side);
        c->side = nullptr;
    }
    if(const char *lim = getenv("SWGB_SPAN_ROWS")) c->spanRowsLimit = strtoull(lim, nullptr, 10);
    // bin lists: SWGB_BIN_LIST entries per bin (0: none), for draws of at
    // least SWGB_BIN_LIST_MIN triangles
    c->binListPerBin = BIN_LIST_DEFAULT;
    c->binListMinTris = BIN_LIST_MIN_TRIANGLES;
    if(const char *lim = getenv("SWGB_BIN_LIST")) c->binListPerBin = (uint32_t)strtoul(lim, nullptr, 10);
    if(const char *lim = getenv("SWGB_BIN_LIST_MIN")) c->binListMinTris = (uint32_t)strtoul(lim, nullptr, 10);
    if((s = cuda_check(cudaMalloc((void **)&c->polyCount, sizeof(uint32_t)), "polyCount")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->spanCount, sizeof(unsigned long long)), "spanCount")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->binQueue, sizeof(unsigned int)), "binQueue")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->counters, CTX_COUNTERS * sizeof(unsigned long long)), "counters")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->error, sizeof(int)), "error")) != SWGB_OK)
    {
        swgb_ctx_destroy(c);
        return s;
    }
    uint16_t lut[256];
    srgb_table(lut);
    if((s = cuda_check(cudaMalloc((void **)&c->srgbLut, sizeof(lut)), "sRGB table")) != SWGB_OK ||
       (s = cuda_check(cudaMemcpy(c->srgbLut, lut, sizeof(lut), cudaMemcpyHostToDevice), "sRGB table")) != SWGB_OK)
    {
        swgb_ctx_destroy(c);
        return s;
    }
    cudaMemset(c->counters, 0, CTX_COUNTERS * sizeof(unsigned long long));
    cudaMemset(c->error, 0, sizeof(int));
    cudaMemset(c->polyCount, 0, sizeof(uint32_t));
    *out = c;
    return SWGB_OK;
}

swgb_status swgb_ctx_destroy(swgb_ctx *c)
{
    if(!c) return SWGB_INVALID_ARG;
    cudaSetDevice(c->device);
    if(c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->ptv);
    cudaFree(c->binDiff);
    cudaFree(c->restart);
    cudaFree(c->srgbLut);
    cudaFree(c->binOrder);
    cudaFree(c->binList);
    cudaFree(c->triBox);
    cudaFree(c->triInfo);
    cudaFree(c->planes);
    cudaFree(c->spans);
    cudaFree(c->spanCount);
    cudaFree(c->chunkBox);
    cudaFree(c->superBox);
    cudaFree(c->poly);
    cudaFree(c->polyCount);
    cudaFree(c->binQueue);
    cudaFree(c->counters);
    cudaFree(c->error);
    if(c->ownStream && c->stream) cudaStreamDestroy(c->stream);
    if(c->side)
    {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    if(c->sideFork) cudaEventDestroy(c->sideFork);
    if(c->sideJoin) cudaEventDestroy(c->sideJoin);
    if(c->evPairs)
        for(auto &p : *c->evPairs)
        {
            cudaEventDestroy(p.second.first);
            cudaEventDestroy(p.second.second);
        }
    if(c->evFree)
        for(auto e : *c->evFree) cudaEventDestroy(e);
    delete c->evPairs;
    delete c->evFree;
    batch_free(c->batch);
    cudaFree(c->adjScratch);
    cudaFree(c->ptv64);
    delete c;
    return SWGB_OK;
}

swgb_status swgb_ctx_set_stream(swgb_ctx *c, void *stream)
{
    if(!c) return SWGB_INVALID_ARG;
    if(c->ownStream && c->stream)
    {
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    c->ownStream = false;
    c->stream = (cudaStream_t)stream;
    return SWGB_OK;
}

swgb_status swgb_draw(swgb_ctx *ctx, const swgb_pipeline_state *st, const swgb_draw_args *args)
{
    if(!ctx || !st || !args) return set_error(SWGB_INVALID_ARG, "null argument");
    DrawParams D;
    swgb_status s = bake(st, args, D);
    if(s != SWGB_OK) return s;
    if(D.count == 0) return SWGB_OK;
    apply_config(ctx, D);
    cudaSetDevice(ctx->device);
    return enqueue(ctx, D, (cudaEvent_t)args->raster_wait_event);
}

// The allocation-free variant of swgb_draw: the same validation, baking and
// kernels, with every scratch buffer carved out of g_noalloc_scratch.  It calls
// no cudaMalloc/cudaFree and no allocating library routine.
swgb_status swgb_draw_noalloc(const swgb_pipeline_state *st, const swgb_draw_args *args, void *stream)
{
    if(!st || !args) return set_error(SWGB_INVALID_ARG, "null argument");
    if(args->restart_index_count && args->index_type != SWGB_INDEX_TYPE_NONE)
        return set_error(SWGB_UNSUPPORTED_STATE, "swgb_draw_noalloc: primitive restart needs swgb_draw");
    if(args->count == 0) return SWGB_OK;
    if(args->count > SWGB_NOALLOC_MAX_TRIANGLES)
        return set_error(SWGB_INVALID_ARG, "swgb_draw_noalloc: more than SWGB_NOALLOC_MAX_TRIANGLES (32768) triangles");
    DrawParams D;
    swgb_status s = bake(st, args, D);
    if(s != SWGB_OK) return s;
    if(D.ms > 1) return set_error(SWGB_UNSUPPORTED_STATE, "swgb_draw_noalloc: multisampled attachments need swgb_draw");
    if(D.texSRGB) return set_error(SWGB_UNSUPPORTED_STATE, "swgb_draw_noalloc: sRGB textures need swgb_draw");
    if(D.vertexCount > SWGB_NOALLOC_MAX_VERTICES)
        return set_error(SWGB_INVALID_ARG, "swgb_draw_noalloc: vertex_count above SWGB_NOALLOC_MAX_VERTICES (98304)");
    int dev = 0;
    if((s = cuda_check(cudaGetDevice(&dev), "cudaGetDevice")) != SWGB_OK) return s;
    NoAllocDevice *nd = nullptr;
    if((s = noalloc_device(dev, nd)) != SWGB_OK) return s;
    unsigned char *b = nd->base;
    D.ptv = (float4 *)(b + NA_OFF_PTV);
    D.triBox = (short4 *)(b + NA_OFF_BOX);
    D.triInfo = (TriInfo *)(b + NA_OFF_INFO);
    D.planes = (float4 *)(b + NA_OFF_PLANES);
    D.chunkBox = (short4 *)(b + NA_OFF_CHUNK);
    D.superBox = (int4 *)(b + NA_OFF_SUPER);
    D.spans = (uint32_t *)(b + NA_OFF_SPANS);
    D.spanCapacity = NA_SPAN_ROWS;
    D.poly = (int2 *)(b + NA_OFF_POLY);
    D.polyCapacity = NA_TRIS;
    unsigned char *w = b + NA_OFF_WORDS;
    D.counters = (unsigned long long *)w;
    D.spanCount = (unsigned long long *)(w + 64);
    D.polyCount = (uint32_t *)(w + 72);
    D.binQueue = (unsigned int *)(w + 76);
    D.error = (int *)(w + 80);
    cudaStream_t st0 = (cudaStream_t)stream;
    if(args->raster_wait_event) cudaStreamWaitEvent(st0, (cudaEvent_t)args->raster_wait_event, 0);
    // The array keeps the previous call's contents: the counters and the error
    // word are cleared here, the queue heads and super-chunk boxes by k_vertex.
    if((s = cuda_check(cudaMemsetAsync(w, 0, NA_WORDS_BYTES, st0), "clear scratch words")) != SWGB_OK) return s;
    const uint32_t nv = D.vertexCount;
    k_vertex<<<(nv + 255) / 256, 256, 0, st0>>>(D, nv);
    const uint32_t setupBlocks = (uint32_t)((D.count + SETUP_THREADS - 1) / SETUP_THREADS);
    k_setup<<<setupBlocks, SETUP_THREADS, 0, st0>>>(D);
    if(D.binsX > 0 && D.binsY > 0)
    {
        uint32_t blocks = (uint32_t)((D.binsX * D.binsY + RASTER_WARPS - 1) / RASTER_WARPS);
        const int v = raster_variant(D);  // a single-sample 16x16 variant
        if(blocks > (uint32_t)nd->rasterBlocks[v]) blocks = (uint32_t)nd->rasterBlocks[v];
        launch_raster(D, blocks, st0);
    }
    return cuda_check(cudaGetLastError(), "kernel launch");
}

swgb_status swgb_draw_batch(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n)
{
    if(!ctx || (!states && n) || (!args && n)) return set_error(SWGB_INVALID_ARG, "null argument");
    if(n == 0) return SWGB_OK;
    cudaSetDevice(ctx->device);
    for(uint32_t i = 0; i < n; i++)
        if(args[i].raster_wait_event) cudaStreamWaitEvent(ctx->stream, (cudaEvent_t)args[i].raster_wait_event, 0);
    return draw_batch(ctx, states, args, n);
}

swgb_status swgb_ctx_set_raster_config(swgb_ctx *ctx, const swgb_raster_config *config)
{
    if(!ctx || !config) return set_error(SWGB_INVALID_ARG, "null argument");
    if(shape_index((int)config->bin_width, (int)config->bin_height) < 0) return set_error(SWGB_INVALID_ARG, "unsupported bin shape");
    if(config->hiz > 1) return set_error(SWGB_INVALID_ARG, "hiz must be 0 or 1");
    ctx->rasterConfig = *config;
    ctx->rasterConfig.reserved = 0;
    return SWGB_OK;
}

swgb_status swgb_ctx_get_raster_config(swgb_ctx *ctx, swgb_raster_config *config)
{
    if(!ctx || !config) return set_error(SWGB_INVALID_ARG, "null argument");
    *config = ctx->rasterConfig;
    return SWGB_OK;
}

swgb_status swgb_autotune(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n, int batched,
                          uint32_t runs, swgb_raster_config *best, swgb_raster_config *candidates, double *ms, double *ms_min,
                          double *ms_max)
{
    if(!ctx || (n && (!states || !args))) return set_error(SWGB_INVALID_ARG, "null argument");
    if(runs == 0) runs = SWGB_AUTOTUNE_DEFAULT_RUNS;
    if(runs > SWGB_AUTOTUNE_MAX_RUNS) return set_error(SWGB_INVALID_ARG, "swgb_autotune: runs above SWGB_AUTOTUNE_MAX_RUNS");
    cudaSetDevice(ctx->device);
    for(uint32_t i = 0; i < n; i++)  // textures still arriving: wait before the first run
        if(args[i].raster_wait_event) cudaStreamWaitEvent(ctx->stream, (cudaEvent_t)args[i].raster_wait_event, 0);
    // Validate every draw first (bake has no side effects), and collect the
    // attachment byte ranges the draws can touch: every row of every sample
    // plane of the colour and depth attachments, merged.
    std::vector<std::pair<uintptr_t, uintptr_t>> iv;
    for(uint32_t i = 0; i < n; i++)
    {
        DrawParams D;
        swgb_status s = bake(&states[i], &args[i], D);
        if(s != SWGB_OK) return s;
        if(D.count == 0) continue;
        if(batched && D.restart) return set_error(SWGB_UNSUPPORTED_STATE, "swgb_draw_batch: primitive restart needs swgb_draw");
        const swgb_pipeline_state &st = states[i];
        const uint32_t h = st.framebuffer_height;
        const size_t cRow = (size_t)st.framebuffer_width * 4 * color_words(D.cf);
        for(int q = 0; q < D.ms; q++)
        {
            const uintptr_t c = (uintptr_t)st.color + (uintptr_t)q * D.colorSlice;
            iv.push_back({c, c + (uintptr_t)(h - 1) * st.color_pitch_bytes + cRow});
            if(D.stencilTest)
            {
                const uintptr_t sb = (uintptr_t)st.stencil + (uintptr_t)q * D.stencilSlice;
                iv.push_back({sb, sb + (uintptr_t)(h - 1) * st.stencil_pitch_bytes + st.framebuffer_width});
            }
            if(st.depth)
            {
                const uintptr_t d = (uintptr_t)st.depth + (uintptr_t)q * D.depthSlice;
                iv.push_back({d, d + (uintptr_t)(h - 1) * st.depth_pitch_bytes + (size_t)st.framebuffer_width * (D.depth16 ? 2 : 4)});
            }
        }
    }
    std::sort(iv.begin(), iv.end());
    std::vector<std::pair<uintptr_t, uintptr_t>> merged;
    for(const auto &r : iv)
    {
        if(!merged.empty() && r.first <= merged.back().second) merged.back().second = std::max(merged.back().second, r.second);
        else merged.push_back(r);
    }
    size_t total = 0;
    for(const auto &r : merged) total += r.second - r.first;

    swgb_raster_config cands[SWGB_AUTOTUNE_CANDIDATES];
    for(int k = 0; k < SWGB_AUTOTUNE_CANDIDATES; k++)
        cands[k] = {(uint32_t)SHAPE_W[k >> 1], (uint32_t)SHAPE_H[k >> 1], (k & 1) ? 0u : 1u, 0u};
    static_assert(SWGB_AUTOTUNE_CANDIDATES == 2 * NSHAPES, "one candidate per bin shape and hiz setting");

    uint8_t *save = nullptr;
    unsigned long long *cntSave = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const swgb_raster_config prev = ctx->rasterConfig;
    const bool timing = ctx->timing;
    ctx->timing = false;  // time the production path (graph replays), not the per-kernel one
    swgb_status s = SWGB_OK;
    auto restore = [&]() -> swgb_status {
        size_t off = 0;
        for(const auto &r : merged)
        {
            swgb_status t = cuda_check(cudaMemcpyAsync((void *)r.first, save + off, r.second - r.first, cudaMemcpyDeviceToDevice, ctx->stream),
                                       "autotune restore");
            if(t != SWGB_OK) return t;
            off += r.second - r.first;
        }
        return SWGB_OK;
    };
    auto run = [&]() -> swgb_status {
        if(batched) return n ? draw_batch(ctx, states, args, n) : SWGB_OK;
        for(uint32_t i = 0; i < n; i++)
        {
            DrawParams D;
            swgb_status t = bake(&states[i], &args[i], D);
            if(t != SWGB_OK) return t;
            if(D.count == 0) continue;
            apply_config(ctx, D);
            if((t = enqueue(ctx, D)) != SWGB_OK) return t;
        }
        return SWGB_OK;
    };
    double t[SWGB_AUTOTUNE_CANDIDATES] = {}, tMin[SWGB_AUTOTUNE_CANDIDATES] = {}, tMax[SWGB_AUTOTUNE_CANDIDATES] = {};
    int bestK = 0;
    do
    {
        if(total && (s = cuda_check(cudaMalloc((void **)&save, total), "autotune attachment copy")) != SWGB_OK) break;
        if((s = cuda_check(cudaMalloc((void **)&cntSave, CTX_COUNTERS * sizeof(unsigned long long)), "autotune counters")) != SWGB_OK) break;
        if((s = cuda_check(cudaEventCreate(&e0), "event")) != SWGB_OK || (s = cuda_check(cudaEventCreate(&e1), "event")) != SWGB_OK) break;
        size_t off = 0;
        for(const auto &r : merged)
        {
            if((s = cuda_check(cudaMemcpyAsync(save + off, (const void *)r.first, r.second - r.first, cudaMemcpyDeviceToDevice, ctx->stream),
                               "autotune save")) != SWGB_OK)
                break;
            off += r.second - r.first;
        }
        if(s != SWGB_OK) break;
        if((s = cuda_check(cudaMemcpyAsync(cntSave, ctx->counters, CTX_COUNTERS * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, ctx->stream),
                           "autotune counters")) != SWGB_OK)
            break;
        for(int k = 0; k < SWGB_AUTOTUNE_CANDIDATES && s == SWGB_OK; k++)
        {
            ctx->rasterConfig = cands[k];
            double samples[SWGB_AUTOTUNE_MAX_RUNS];
            // run 0 warms up (module load, scratch growth, graph capture);
            // runs 1..runs are timed one at a time
            for(uint32_t rep = 0; rep <= runs && s == SWGB_OK; rep++)
            {
                if((s = restore()) != SWGB_OK) break;
                // the counters end as one run of the draws left them
                if((s = cuda_check(cudaMemcpyAsync(ctx->counters, cntSave, CTX_COUNTERS * sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                                                   ctx->stream), "autotune counters")) != SWGB_OK)
                    break;
                if(rep > 0) cudaEventRecord(e0, ctx->stream);
                if((s = run()) != SWGB_OK) break;
                if(rep == 0) continue;
                cudaEventRecord(e1, ctx->stream);
                float el = 0.0f;
                if((s = cuda_check(cudaEventSynchronize(e1), "autotune sync")) != SWGB_OK) break;
                cudaEventElapsedTime(&el, e0, e1);
                samples[rep - 1] = el;
            }
            if(s != SWGB_OK) break;
            std::sort(samples, samples + runs);
            t[k] = (runs & 1) ? samples[runs / 2] : 0.5 * (samples[runs / 2 - 1] + samples[runs / 2]);
            tMin[k] = samples[0];
            tMax[k] = samples[runs - 1];
            if(t[k] < t[bestK]) bestK = k;
        }
    } while(false);
    if(s == SWGB_OK) s = cuda_check(cudaStreamSynchronize(ctx->stream), "autotune sync");
    if(save) cudaFree(save);
    if(cntSave) cudaFree(cntSave);
    if(e0) cudaEventDestroy(e0);
    if(e1) cudaEventDestroy(e1);
    ctx->timing = timing;
    if(s != SWGB_OK)
    {
        ctx->rasterConfig = prev;
        return s;
    }
    ctx->rasterConfig = cands[bestK];
    if(best) *best = cands[bestK];
    for(int k = 0; k < SWGB_AUTOTUNE_CANDIDATES; k++)
    {
        if(candidates) candidates[k] = cands[k];
        if(ms) ms[k] = t[k];
        if(ms_min) ms_min[k] = tMin[k];
        if(ms_max) ms_max[k] = tMax[k];
    }
    return SWGB_OK;
}

swgb_status swgb_plan_batch(const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n, uint32_t *segment_first,
                            uint32_t *segment_count)
{
    if((n && (!states || !args)) || !segment_count) return set_error(SWGB_INVALID_ARG, "null argument");
    std::vector<DrawParams> draws;
    std::vector<uint32_t> src;
    for(uint32_t i = 0; i < n; i++)
    {
        if(args[i].count == 0 && !args[i].restart_index_count) continue;
        DrawParams D;
        swgb_status s = bake(&states[i], &args[i], D);
        if(s != SWGB_OK) return s;
        if(D.restart) return set_error(SWGB_UNSUPPORTED_STATE, "swgb_draw_batch: primitive restart needs swgb_draw");
        draws.push_back(D);
        src.push_back(i);
    }
    std::vector<std::pair<uint32_t, uint32_t>> segs;
    if(!draws.empty()) segment_batch(draws, src, states, args, segs);
    if(segment_first)
        for(size_t k = 0; k < segs.size(); k++) segment_first[k] = src[segs[k].first];
    *segment_count = (uint32_t)segs.size();
    return SWGB_OK;
}

swgb_status swgb_draw_adjoint(swgb_ctx *ctx, const swgb_pipeline_state *state, const swgb_draw_args *args, const swgb_adjoint_args *adj)
{
    if(!ctx || !state || !args || !adj) return set_error(SWGB_INVALID_ARG, "null argument");
    cudaSetDevice(ctx->device);
    return draw_adjoint(ctx, state, args, adj);
}

swgb_status swgb_draw_adjoint_batch(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args,
                                    const swgb_adjoint_args *adjs, uint32_t n)
{
    if(!ctx || (n && (!states || !args || !adjs))) return set_error(SWGB_INVALID_ARG, "null argument");
    if(n == 0) return SWGB_OK;
    cudaSetDevice(ctx->device);
    return draw_adjoint_batch(ctx, states, args, adjs, n);
}

// --------------------------------------------------------------------------
// Blitter: clears, resolves, blits (kernels in swgb_blit.cu)
// --------------------------------------------------------------------------

namespace {

struct BlitFormat {
    bool colour;  // a colour format of the Blitter kernels
    int kind;     // swgbb::BK_*
    bool srgb;
    int bytes;
};

BlitFormat blit_format(uint32_t f)
{
    switch(f)
    {
    case SWGB_FORMAT_R8G8B8A8_UNORM: return {true, swgbb::BK_RGBA8, false, 4};
    case SWGB_FORMAT_R8G8B8A8_SRGB: return {true, swgbb::BK_RGBA8, true, 4};
    case SWGB_FORMAT_B8G8R8A8_UNORM: return {true, swgbb::BK_BGRA8, false, 4};
    case SWGB_FORMAT_B8G8R8A8_SRGB: return {true, swgbb::BK_BGRA8, true, 4};
    case SWGB_FORMAT_R16G16B16A16_SFLOAT: return {true, swgbb::BK_RGBA16F, false, 8};
    case SWGB_FORMAT_R32G32B32A32_SFLOAT: return {true, swgbb::BK_RGBA32F, false, 16};
    case SWGB_FORMAT_D32_SFLOAT: return {false, -1, false, 4};
    case SWGB_FORMAT_D16_UNORM: return {false, -1, false, 2};
    case SWGB_FORMAT_S8_UINT: return {false, -1, false, 1};
    default: return {false, -1, false, 0};
    }
}

constexpr uint32_t MAX_IMAGE_DIM = 16384;  // vk::MAX_IMAGE_LEVELS_2D = 15 levels

swgb_status check_image(const swgb_image *im, const char *what)
{
    const BlitFormat f = blit_format(im ? im->format : 0);
    if(!im || !im->data) return set_error(SWGB_INVALID_ARG, what);
    if(f.bytes == 0) return set_error(SWGB_UNSUPPORTED_STATE, "blitter: image format");
    if(im->width == 0 || im->height == 0 || im->width > MAX_IMAGE_DIM || im->height > MAX_IMAGE_DIM)
        return set_error(SWGB_INVALID_ARG, "blitter: image extent");
    if(im->samples != 1 && im->samples != 4) return set_error(SWGB_UNSUPPORTED_STATE, "blitter: sample count");
    const uint64_t b = (uint64_t)f.bytes;
    if((uintptr_t)im->data % b || im->pitch_bytes % b || im->pitch_bytes < (uint64_t)im->width * b)
        return set_error(SWGB_INVALID_ARG, "blitter: image base and row pitch must be texel-aligned, pitch >= width");
    if(im->samples > 1 && (im->slice_bytes % b || im->slice_bytes < im->pitch_bytes * im->height))
        return set_error(SWGB_INVALID_ARG, "blitter: sample-plane pitch");
    return SWGB_OK;
}

}  // namespace

swgb_status swgb_clear(swgb_ctx *ctx, const void *value, uint32_t value_format, const swgb_image *dst, const swgb_rect *area)
{
    if(!ctx || !value) return set_error(SWGB_INVALID_ARG, "null argument");
    swgb_status s;
    if((s = check_image(dst, "clear: dst")) != SWGB_OK) return s;
    const BlitFormat f = blit_format(dst->format);
    const uint32_t need = f.colour ? SWGB_FORMAT_R32G32B32A32_SFLOAT
                          : dst->format == SWGB_FORMAT_S8_UINT ? SWGB_FORMAT_S8_UINT : SWGB_FORMAT_D32_SFLOAT;
    if(value_format != need) return set_error(SWGB_INVALID_ARG, "clear: value format does not match the image");
    swgb_rect a = area ? *area : swgb_rect{0, 0, dst->width, dst->height};
    if(a.x < 0 || a.y < 0 || (uint64_t)a.x + a.width > dst->width || (uint64_t)a.y + a.height > dst->height)
        return set_error(SWGB_INVALID_ARG, "clear: area outside the image");
    if(a.width == 0 || a.height == 0) return SWGB_OK;
    swgbb::ClearParams C = {};
    C.dst = (uint8_t *)dst->data;
    C.pitch = (int64_t)dst->pitch_bytes;
    C.slice = (int64_t)dst->slice_bytes;
    C.x = a.x;
    C.y = a.y;
    C.rows = (int)a.height;
    C.planes = (int)dst->samples;
    C.rowBytes = (int64_t)a.width * f.bytes;
    C.bpp = f.bytes;
    C.dstFormat = dst->format;
    C.dstKind = f.kind;
    C.dstSRGB = f.srgb;
    // normalized formats clamp the value (Blitter.cpp:64-85)
    C.normalized = (f.colour && f.kind != swgbb::BK_RGBA16F && f.kind != swgbb::BK_RGBA32F) || dst->format == SWGB_FORMAT_D16_UNORM;
    if(value_format == SWGB_FORMAT_S8_UINT)
        memcpy(&C.stencil, value, 4);
    else
        memcpy(C.value, value, value_format == SWGB_FORMAT_D32_SFLOAT ? 4 : 16);
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaSuccess;
    timed_launch(ctx, SWGB_KERNEL_BLIT, [&] { e = swgbb::launch_clear(C, ctx->stream); });
    return cuda_check(e, "clear launch");
}

namespace {

// Blitter::blit's setup (Blitter.cpp:1820-1895) of a 2D region, src samples
// included (a resolve that misses the fast path is a NEAREST blit).
swgb_status enqueue_blit(swgb_ctx *ctx, const swgb_image *src, const swgb_image *dst, swgb_blit_region r, bool filter)
{
    const BlitFormat sf = blit_format(src->format), df = blit_format(dst->format);
    if(!sf.colour || !df.colour) return set_error(SWGB_UNSUPPORTED_STATE, "blit: colour formats only");
    if(r.dst[0] > r.dst[2])
    {
        std::swap(r.src[0], r.src[2]);
        std::swap(r.dst[0], r.dst[2]);
    }
    if(r.dst[1] > r.dst[3])
    {
        std::swap(r.src[1], r.src[3]);
        std::swap(r.dst[1], r.dst[3]);
    }
    if(r.dst[0] < 0 || r.dst[1] < 0 || (uint32_t)r.dst[2] > dst->width || (uint32_t)r.dst[3] > dst->height)
        return set_error(SWGB_INVALID_ARG, "blit: destination region outside the image");
    if(r.dst[0] == r.dst[2] || r.dst[1] == r.dst[3]) return SWGB_OK;
    const float widthRatio = static_cast<float>(r.src[2] - r.src[0]) / static_cast<float>(r.dst[2] - r.dst[0]);
    const float heightRatio = static_cast<float>(r.src[3] - r.src[1]) / static_cast<float>(r.dst[3] - r.dst[1]);
    const float x0 = r.src[0] + (0.5f - r.dst[0]) * widthRatio;
    const float y0 = r.src[1] + (0.5f - r.dst[1]) * heightRatio;
    swgbb::BlitParams P = {};
    P.src = (const uint8_t *)src->data;
    P.dst = (uint8_t *)dst->data;
    P.sPitch = (int64_t)src->pitch_bytes;
    P.sSlice = (int64_t)src->slice_bytes;
    P.dPitch = (int64_t)dst->pitch_bytes;
    P.srcKind = sf.kind;
    P.dstKind = df.kind;
    P.sBytes = sf.bytes;
    P.dBytes = df.bytes;
    P.srcSRGB = sf.srgb;
    P.dstSRGB = df.srgb;
    P.srcSamples = (int)src->samples;
    P.filter = filter;
    P.allowSRGB = filter || src->samples > 1 || sf.srgb != df.srgb;
    P.clampToEdge = r.src[0] < 0 || r.src[1] < 0 || (uint32_t)r.src[2] > src->width || (uint32_t)r.src[3] > src->height ||
                    (filter && (x0 < 0.5f || y0 < 0.5f));
    P.x0 = x0;
    P.y0 = y0;
    P.w = widthRatio;
    P.h = heightRatio;
    P.x0d = r.dst[0];
    P.x1d = r.dst[2];
    P.y0d = r.dst[1];
    P.y1d = r.dst[3];
    P.sW = (int)src->width;
    P.sH = (int)src->height;
    P.vec16 = (uintptr_t)src->data % 16 == 0 && src->pitch_bytes % 16 == 0;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaSuccess;
    timed_launch(ctx, SWGB_KERNEL_BLIT, [&] { e = swgbb::launch_blit(P, ctx->stream); });
    return cuda_check(e, "blit launch");
}

}  // namespace

swgb_status swgb_resolve(swgb_ctx *ctx, const swgb_image *src, const swgb_image *dst, const swgb_resolve_region *region)
{
    if(!ctx) return set_error(SWGB_INVALID_ARG, "null argument");
    swgb_status s;
    if((s = check_image(src, "resolve: src")) != SWGB_OK || (s = check_image(dst, "resolve: dst")) != SWGB_OK) return s;
    if(src->format != dst->format || !blit_format(src->format).colour)
        return set_error(SWGB_INVALID_ARG, "resolve: src and dst must have the same colour format");
    if(src->samples != 4 || dst->samples != 1) return set_error(SWGB_INVALID_ARG, "resolve: 4-sample src into single-sample dst");
    swgb_resolve_region r = region ? *region : swgb_resolve_region{0, 0, 0, 0, src->width, src->height};
    if(r.src_x < 0 || r.src_y < 0 || r.dst_x < 0 || r.dst_y < 0 || (uint64_t)r.src_x + r.width > src->width ||
       (uint64_t)r.src_y + r.height > src->height || (uint64_t)r.dst_x + r.width > dst->width ||
       (uint64_t)r.dst_y + r.height > dst->height)
        return set_error(SWGB_INVALID_ARG, "resolve: region outside an image");
    if(r.width == 0 || r.height == 0) return SWGB_OK;
    // fastResolve (Blitter.cpp:2079-2205): whole images, R8G8B8A8_UNORM / B8G8R8A8_UNORM
    const bool whole = r.src_x == 0 && r.src_y == 0 && r.dst_x == 0 && r.dst_y == 0 && r.width == src->width &&
                       r.height == src->height && src->width == dst->width && src->height == dst->height;
    if(whole && (src->format == SWGB_FORMAT_R8G8B8A8_UNORM || src->format == SWGB_FORMAT_B8G8R8A8_UNORM))
    {
        swgbb::ResolveParams R = {};
        R.src = (const uint8_t *)src->data;
        R.dst = (uint8_t *)dst->data;
        R.sPitch = (int64_t)src->pitch_bytes;
        R.sSlice = (int64_t)src->slice_bytes;
        R.dPitch = (int64_t)dst->pitch_bytes;
        R.width = (int)r.width;
        R.height = (int)r.height;
        R.vec16 = (uintptr_t)src->data % 16 == 0 && (uintptr_t)dst->data % 16 == 0 && src->pitch_bytes % 16 == 0 &&
                  dst->pitch_bytes % 16 == 0 && src->slice_bytes % 16 == 0;
        cudaSetDevice(ctx->device);
        cudaError_t e = cudaSuccess;
        timed_launch(ctx, SWGB_KERNEL_BLIT, [&] { e = swgbb::launch_resolve_bytes(R, ctx->stream); });
        return cuda_check(e, "resolve launch");
    }
    // otherwise a NEAREST blit of the region, which averages the samples (Blitter.cpp:2052-2072)
    swgb_blit_region b;
    b.src[0] = r.src_x;
    b.src[1] = r.src_y;
    b.src[2] = r.src_x + (int32_t)r.width;
    b.src[3] = r.src_y + (int32_t)r.height;
    b.dst[0] = r.dst_x;
    b.dst[1] = r.dst_y;
    b.dst[2] = r.dst_x + (int32_t)r.width;
    b.dst[3] = r.dst_y + (int32_t)r.height;
    return enqueue_blit(ctx, src, dst, b, false);
}

swgb_status swgb_blit(swgb_ctx *ctx, const swgb_image *src, const swgb_image *dst, const swgb_blit_region *region, uint32_t filter)
{
    if(!ctx || !region) return set_error(SWGB_INVALID_ARG, "null argument");
    swgb_status s;
    if((s = check_image(src, "blit: src")) != SWGB_OK || (s = check_image(dst, "blit: dst")) != SWGB_OK) return s;
    if(src->samples != 1 || dst->samples != 1) return set_error(SWGB_INVALID_ARG, "blit: single-sample images only");
    if(filter != SWGB_FILTER_NEAREST && filter != SWGB_FILTER_LINEAR) return set_error(SWGB_INVALID_ARG, "blit: filter");
    return enqueue_blit(ctx, src, dst, *region, filter == SWGB_FILTER_LINEAR);
}

swgb_status swgb_sync(swgb_ctx *ctx)
{
    if(!ctx) return SWGB_INVALID_ARG;
    swgb_status s = cuda_check(cudaStreamSynchronize(ctx->stream), "stream sync");
    if(s != SWGB_OK) return s;
    int err = 0;
    if((s = cuda_check(cudaMemcpy(&err, ctx->error, sizeof(int), cudaMemcpyDeviceToHost), "error word")) != SWGB_OK) return s;
    if(err)
    {
        cudaMemset(ctx->error, 0, sizeof(int));
        if(err & ERR_INDEX_RANGE) return set_error(SWGB_INVALID_ARG, "an index was >= vertex_count; its triangle was dropped");
        return set_error(SWGB_DEVICE_ERROR, "clipped-polygon scratch overflow");
    }
    return SWGB_OK;
}

swgb_status swgb_get_counters(swgb_ctx *ctx, swgb_counters *out)
{
    if(!ctx || !out) return SWGB_INVALID_ARG;
    swgb_status s = cuda_check(cudaStreamSynchronize(ctx->stream), "stream sync");
    if(s != SWGB_OK) return s;
    unsigned long long h[CTX_COUNTERS];
    if((s = cuda_check(cudaMemcpy(h, ctx->counters, sizeof(h), cudaMemcpyDeviceToHost), "counters")) != SWGB_OK) return s;
    out->triangles_in = h[0];
    out->triangles_rejected = h[1];
    out->triangles_clipped = h[2];
    out->triangles_visible = h[3];
    out->quads = h[4];
    out->fragments_tested = h[5];
    out->fragments_passed = h[6];
    out->texture_levels_mask = h[7];
    out->adjoint_fragments = h[CNT_ADJ_FRAGMENTS];
    out->adjoint_depth_mismatch = h[CNT_ADJ_MISMATCH];
    out->adjoint_list_overflow = h[CNT_ADJ_OVERFLOW];
    out->reserved = 0;
    return SWGB_OK;
}

swgb_status swgb_reset_counters(swgb_ctx *ctx)
{
    if(!ctx) return SWGB_INVALID_ARG;
    return cuda_check(cudaMemsetAsync(ctx->counters, 0, CTX_COUNTERS * sizeof(unsigned long long), ctx->stream), "counters reset");
}

uint64_t swgb_launch_count(swgb_ctx *ctx) { return ctx ? ctx->launches : 0; }

swgb_status swgb_set_kernel_timing(swgb_ctx *ctx, int enable)
{
    if(!ctx) return SWGB_INVALID_ARG;
    ctx->timing = enable != 0;
    ctx->timingKinds = (enable & 0x10000) ? (uint32_t)(enable & 0xFFFF) : 0xFFFFu;
    return SWGB_OK;
}

swgb_status swgb_get_kernel_times(swgb_ctx *ctx, double ms[SWGB_KERNEL_KINDS], uint32_t launches[SWGB_KERNEL_KINDS])
{
    if(!ctx || !ms || !launches) return SWGB_INVALID_ARG;
    swgb_status s = cuda_check(cudaStreamSynchronize(ctx->stream), "stream sync");
    if(s != SWGB_OK) return s;
    for(int k = 0; k < SWGB_KERNEL_KINDS; k++) { ms[k] = 0.0; launches[k] = 0; }
    for(auto &p : *ctx->evPairs)
    {
        float t = 0.0f;
        cudaEventElapsedTime(&t, p.second.first, p.second.second);
        if(p.first >= 0 && p.first < SWGB_KERNEL_KINDS)
        {
            ms[p.first] += t;
            launches[p.first]++;
        }
        ctx->evFree->push_back(p.second.first);
        ctx->evFree->push_back(p.second.second);
    }
    ctx->evPairs->clear();
    return SWGB_OK;
}

}  // extern "C"
