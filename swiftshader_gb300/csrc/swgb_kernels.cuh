// swgb_kernels.cuh -- device code of the draw hot path (sm_103a), shared by
// the translation units of libswgb: swgb_draw.cu (vertex, setup, binning and
// adjoint kernels, host side, C-ABI) and swgb_raster.cu (the raster kernel variants,
// compiled once per colour format and linked into the same library).
// SWGB_RASTER_TU leaves out everything but the raster stage.
#ifndef SWGB_KERNELS_CUH
#define SWGB_KERNELS_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/swgb.h"
#include "swgb_numeric.cuh"

namespace swgbk {

using namespace swgb;

constexpr int MAXV = 7;          // varying components carried per vertex
constexpr int BIN = 16;          // bin side in pixels; one warp owns one bin
constexpr int RASTER_WARPS = 4;  // independent warps (bins) per raster block
constexpr int RASTER_THREADS = 32 * RASTER_WARPS;
constexpr int BATCH = 32;        // triangles staged per batch: one per lane
constexpr int SUPER = 64;        // chunks per super-chunk box
constexpr int SETUP_THREADS = 256;
constexpr int CHUNK = 32;        // triangles per chunk box (one setup warp)
constexpr int MAX_POLY = 16;     // clipped polygon capacity (Polygon::B, src/Device/Polygon.hpp:45)

// Bin shapes the raster kernels are built for (width x height in pixels); the
// first is the default and the only one for four-sample draws.  Each shape is
// built with and without hierarchical depth rejection, for every colour format.
constexpr int NSHAPES = 3;
constexpr int SHAPE_W[NSHAPES] = {16, 32, 32};
constexpr int SHAPE_H[NSHAPES] = {16, 16, 32};
constexpr int NRASTER = NSHAPES * 2 * 4 + 2 * 4 + 4 * 4;  // see raster_index
inline int shape_index(int w, int h)
{
    for(int i = 0; i < NSHAPES; i++)
        if(SHAPE_W[i] == w && SHAPE_H[i] == h) return i;
    return -1;
}

enum { CLIP_RIGHT = 1 << 0, CLIP_TOP = 1 << 1, CLIP_FAR = 1 << 2, CLIP_LEFT = 1 << 3,
       CLIP_BOTTOM = 1 << 4, CLIP_NEAR = 1 << 5, CLIP_FRUSTUM = 0x3F, CLIP_FINITE = 1 << 7 };

enum { OP_ZERO_EXT = 1000, OP_SRC_EXT = 1001, OP_DST_EXT = 1002 };

// 4x MSAA sample positions (src/Pipeline/Constants.hpp:26-52, Constants.cpp:293-294):
// VkSampleLocations4 relative to the pixel centre, and in sub-pixel fixed point.
__device__ constexpr float SLX[4] = {0.375f - 0.5f, 0.875f - 0.5f, 0.125f - 0.5f, 0.625f - 0.5f};
__device__ constexpr float SLY[4] = {0.125f - 0.5f, 0.375f - 0.5f, 0.625f - 0.5f, 0.875f - 0.5f};
__device__ constexpr int XF[4] = {-32, 96, -96, 32};
__device__ constexpr int YF[4] = {-96, -32, 32, 96};
constexpr int Y_MIN_MS_OFFSET = 159;  // 256 - toFixedPoint(0.375) - 1
constexpr int Y_MAX_MS_OFFSET = 351;  // 256 + toFixedPoint(0.375) - 1

enum { ERR_INDEX_RANGE = 1, ERR_POLY_OVERFLOW = 2 };

// Device counter words of a context: 0-7 as swgb_counters, then the adjoint's.
enum { CNT_ADJ_FRAGMENTS = 8, CNT_ADJ_MISMATCH = 9, CNT_ADJ_OVERFLOW = 10, CTX_COUNTERS = 12 };

struct TexLevel {
    const uint8_t *buf;
    uint32_t w, h, pitch;
    uint32_t uHalf, vHalf;
};

// Per-triangle record written by k_setup next to its pixel box (a short4
// x0, y0, x1, y1 with y0/y1 the trimmed [yMin, yMax); x0 >= x1 = no primitive).
struct TriInfo {
    uint32_t info;     // bits 0-4: polygon vertex count, bit 5: winding d, bit 6: clipped, bit 7: spans stored, bit 8: front-facing
    uint32_t slot;     // clipped polygon slot
    uint32_t spanOff;  // span-buffer index of row y0 of sample 0 (when stored)
    uint32_t rows;     // rows per sample plane in the span buffer
};

// Everything a draw's kernels read, baked on the host from the pipeline state
// (the analog of sw::DrawData plus the processors' state hashes).
struct DrawParams {
    // vertex input
    const uint8_t *vbuf[SWGB_MAX_ATTRIBS];
    uint32_t vstride[SWGB_MAX_ATTRIBS];
    uint32_t voff[SWGB_MAX_ATTRIBS];
    uint32_t vcomp[SWGB_MAX_ATTRIBS];
    int nattr;
    int nv;
    float mvp[16];
    const void *indices;
    uint32_t indexType;
    uint32_t topology;     // SWGB_TOPOLOGY_TRIANGLE_LIST / STRIP / FAN
    int provokingLast;     // VK_PROVOKING_VERTEX_MODE_LAST_VERTEX_EXT
    int restart;           // primitive restart: triangle slots are index positions
    uint32_t restartValue; // all ones of the index type
    const uint32_t *restartLocal;  // per index position: block-local segment start (k_restart_blocks)
    const uint32_t *restartCarry;  // per block of RESTART_BLOCK positions: segment start carried in
    uint32_t firstVertex;
    int32_t baseVertex;
    uint32_t vertexCount;  // post-transform vertices
    uint32_t count;        // triangles
    // DrawData
    float WxF, HxF, X0xF, Y0xF, depthRange, depthNear;
    int sx0, sx1, sy0, sy1;
    int depthClip;
    uint32_t cullMode, frontFace;
    // pixel state
    int depthTest, depthWrite, compareOp;
    int hiz;      // reject triangle-bin pairs against the bin's depth bound
    float biasConstant, biasSlope, biasClamp;  // depth bias (0: none)
    int depthBias;     // biasConstant or biasSlope nonzero: fragments add the triangle's zBias
    int depthBounds;   // depth bounds test against [minBounds, maxBounds]
    float minBounds, maxBounds;
    // stencil (S8_UINT attachment): [0] front-facing, [1] back-facing state
    uint8_t *stencil;
    uint32_t stencilPitch;
    uint64_t stencilSlice;
    int stencilTest;        // stencil test active
    int stencilWrite;       // some op can change a stored value
    uint32_t sFailOp[2], sPassOp[2], sDepthFailOp[2], sCompareOp[2];
    uint32_t sCompareMask[2], sWriteMask[2], sReference[2];
    int earlyDepthOK;       // depth-failing fragments leave no trace (no stencil op on them): early / hierarchical rejection allowed
    float minDepthClamp, maxDepthClamp;
    int blend;
    uint32_t srcC, dstC, opC, srcA, dstA, opA;
    int blendAlpha;  // SRC_ALPHA / ONE_MINUS_SRC_ALPHA / ADD on colour and alpha
    uint32_t writeMask;
    uint32_t writeBytes;  // UNORM8 attachments: writeMask as a byte mask of the stored texel
    int fs;
    int ms;       // samples per pixel: 1 or 4
    uint64_t colorSlice, depthSlice;  // bytes between sample planes
    int cf;       // colour attachment format, CF_*
    int depth16;   // D16_UNORM depth attachment (else D32_SFLOAT)
    int colorSRGB; // R8G8B8A8_SRGB / B8G8R8A8_SRGB colour attachment
    int texBGRA;   // 8-bit texture stored B8G8R8A8
    int texSRGB;   // 8-bit texture with sRGB-encoded R, G, B (decoded through srgbLut)
    const uint16_t *srgbLut;  // sRGBtoLinearFF_FF00: 8-bit sRGB -> 16-bit linear (0xFF00 = 1.0)
    int texFloat; // 0: R8G8B8A8_UNORM texture (16-bit path), 1: RGBA16F, 2: RGBA32F (fp32 path)
    int border;   // an axis addresses CLAMP_TO_BORDER: every texture takes the fp32 path
    int floatPath;  // texFloat || border
    float borderColor[4];  // the border texel in the fp32 path's units (scaled by 0xFF00 for 8-bit textures)
    uint8_t *color;
    uint32_t colorPitch;
    uint8_t *depth;
    uint32_t depthPitch;
    int vec16;  // attachments allow 16-byte row accesses
    // texture
    TexLevel lv[SWGB_MAX_MIP_LEVELS];
    int levelCount;
    float texW, texH;
    float minLod, maxLod, lodBias;
    int texLinear, mipLinear;
    int texRepeatTrilinear;  // R8G8B8A8_UNORM texture, LINEAR filter, MIPMAP_LINEAR, REPEAT on u and v
    uint32_t addrU, addrV;
    // bins: binW x binH pixels, aligned to the bin shape, covering the scissor
    int binW, binH;
    int binX0, binY0, binsX, binsY;
    int nchunks;
    // scratch
    float4 *ptv;          // 4 x float4 per vertex
    double *ptv64;        // adjoint runs only: clip x, y, w and x/w, y/w in fp64 (6 doubles per vertex), else null
    short4 *triBox;       // pixel box per triangle
    TriInfo *triInfo;
    float4 *planes;       // plane equations per triangle (PLANES_STORED floats), written by setup
    int planeVec4;        // float4s of them in use: (8 + 3 * varyings + 3) / 4
    short4 *chunkBox;     // union of the boxes of CHUNK consecutive triangles
    int4 *superBox;       // union of SUPER consecutive chunk boxes (x0, y0, x1, y1)
    int nsuper;
    unsigned int *binQueue;  // next bin for the persistent raster warps
    int *binDiff;         // single draws: 2D difference array of triangle boxes over the bin grid, (binsY+1) x (binsX+1), or null
    int *binFirst;        // single draws: per bin (binsY x binsX) the first chunk whose box reaches it, or null
    uint32_t *binCost;    // single draws: 2D difference array, like binDiff, of each chunk's triangle area spread
                          // evenly over its box's bins, or null
    uint32_t *binOrder;   // single draws: bins heaviest first (k_bin_order; entry = bin | part << 30, part 1 / 2
                          // the top / bottom half of a split bin; the entry count at [2 x bins]), or null
    uint32_t rasterWarps; // resident raster warps of the draw's variant (the split threshold)
    int binSplit;         // the variant rasterises half bins: the order may split its heaviest bins
    uint32_t *binList;       // single draws: per bin its candidate triangles in primitive order (binListCap each), or null
    uint32_t *binListCount;  // candidates per bin; above binListCap the raster walks the bin itself
    uint32_t binListCap;
    uint32_t *spans;      // left | right << 16 per triangle row
    unsigned long long *spanCount;
    uint64_t spanCapacity;
    int2 *poly;           // MAX_POLY per slot
    uint32_t *polyCount;
    uint32_t polyCapacity;
    unsigned long long *counters;
    int *error;
};

// ------------------------------------------------------------------------
// Vertex stage
// ------------------------------------------------------------------------

__device__ __forceinline__ void read_attrib(const DrawParams &D, int a, uint32_t index, float out[4])
{
    const float *p = (const float *)(D.vbuf[a] + (size_t)index * D.vstride[a] + D.voff[a]);
    out[0] = __ldg(p + 0);
    out[1] = __ldg(p + 1);
    if(D.vcomp[a] == 4)
    {
        out[2] = __ldg(p + 2);
        out[3] = __ldg(p + 3);
    }
    else
    {
        out[2] = 0.0f;
        out[3] = 1.0f;  // readStream: componentCount < 4 -> w = 1 (VertexRoutine.cpp:565)
    }
}

// Post-transform vertex: float4[0] = clip position; float4[1] = (X bits, Y
// bits, clipFlags bits, projected z); float4[2] = (rhw, v0, v1, v2);
// float4[3] = (v3, v4, v5, v6).
__device__ __forceinline__ void vertex_body(const DrawParams &D, uint32_t i)
{
    uint32_t index = (D.indexType == SWGB_INDEX_TYPE_NONE ? D.firstVertex + i : i) + (uint32_t)D.baseVertex;
    float p[4];
    read_attrib(D, 0, index, p);
    // OpMatrixTimesVector (src/Pipeline/SpirvShaderArithmetic.cpp:39-55), column-major.
    float r[4];
#pragma unroll
    for(int row = 0; row < 4; row++)
    {
        float v = D.mvp[row] * p[0];
        v = mul_add(D.mvp[4 + row], p[1], v);
        v = mul_add(D.mvp[8 + row], p[2], v);
        v = mul_add(D.mvp[12 + row], p[3], v);
        r[row] = v;
    }
    float x = r[0], y = r[1], z = r[2], w = r[3];
    // computeClipFlags (VertexRoutine.cpp:116-154)
    int f = 0;
    if(w < x) f |= CLIP_RIGHT;
    if(w < y) f |= CLIP_TOP;
    if(!(-w <= x)) f |= CLIP_LEFT;
    if(!(-w <= y)) f |= CLIP_BOTTOM;
    if(D.depthClip)
    {
        if(w < z) f |= CLIP_FAR;
        if(!(0.0f <= z)) f |= CLIP_NEAR;
    }
    const float maxPos = __int_as_float(0x7F7FFFFF);
    if(fabsf(x) <= maxPos && fabsf(y) <= maxPos && fabsf(z) <= maxPos) f |= CLIP_FINITE;
    // writeCache projection (VertexRoutine.cpp:599-612)
    uint32_t wb = __float_as_uint(w);
    if(w == 0.0f) wb |= 0x3F800000u;
    float rhw = 1.0f / __uint_as_float(wb);
    int32_t X = round_int_clamped(D.X0xF + (x * rhw) * D.WxF);
    int32_t Y = round_int_clamped(D.Y0xF + (y * rhw) * D.HxF);
    float v[MAXV + 1] = {0, 0, 0, 0, 0, 0, 0, 0};
    int k = 0;
    for(int a = 1; a < D.nattr; a++)
    {
        float t[4];
        read_attrib(D, a, index, t);
        for(int c = 0; c < (int)D.vcomp[a] && k < MAXV; c++) v[k++] = t[c];
    }
    float4 *o = D.ptv + (size_t)i * 4;
    o[0] = make_float4(x, y, z, w);
    o[1] = make_float4(__int_as_float(X), __int_as_float(Y), __int_as_float(f), z * rhw);
    o[2] = make_float4(rhw, v[0], v[1], v[2]);
    o[3] = make_float4(v[3], v[4], v[5], v[6]);
    if(D.ptv64)
    {
        // the adjoint's clip coordinates: MVP p in fp64, and the projection
        double c[4];
#pragma unroll
        for(int row = 0; row < 4; row++)
            c[row] = (double)D.mvp[row] * p[0] + (double)D.mvp[4 + row] * p[1] + (double)D.mvp[8 + row] * p[2] +
                     (double)D.mvp[12 + row] * p[3];
        double *o64 = D.ptv64 + (size_t)i * 6;
        o64[0] = c[0];
        o64[1] = c[1];
        o64[2] = c[3];
        o64[3] = c[3] != 0.0 ? c[0] / c[3] : 0.0;
        o64[4] = c[3] != 0.0 ? c[1] / c[3] : 0.0;
        o64[5] = 0.0;
    }
}

#ifndef SWGB_RASTER_TU
__global__ void k_vertex(const __grid_constant__ DrawParams D, uint32_t nverts)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i == 0)
    {
        *D.polyCount = 0;
        *D.spanCount = 0;
        *D.binQueue = 0;
    }
    for(uint32_t j = i; j < (uint32_t)D.nsuper; j += gridDim.x * blockDim.x)
        D.superBox[j] = make_int4(0x7FFFFFFF, 0x7FFFFFFF, (int)0x80000000, (int)0x80000000);
    if(D.binDiff)
        for(uint32_t j = i; j < (uint32_t)((D.binsX + 1) * (D.binsY + 1)); j += gridDim.x * blockDim.x) D.binDiff[j] = 0;
    if(D.binFirst)
        for(uint32_t j = i; j < (uint32_t)(D.binsX * D.binsY); j += gridDim.x * blockDim.x) D.binFirst[j] = 0x7FFFFFFF;
    if(D.binCost)
        for(uint32_t j = i; j < (uint32_t)((D.binsX + 1) * (D.binsY + 1)); j += gridDim.x * blockDim.x) D.binCost[j] = 0u;
    if(i < nverts) vertex_body(D, i);
}

// ------------------------------------------------------------------------
// Setup stage
// ------------------------------------------------------------------------

#endif  // SWGB_RASTER_TU

__device__ __forceinline__ uint32_t fetch_index(const DrawParams &D, uint32_t k)
{
    if(D.indexType == SWGB_INDEX_TYPE_NONE) return k;
    if(D.indexType == SWGB_INDEX_TYPE_UINT16) return __ldg((const uint16_t *)D.indices + k);
    if(D.indexType == SWGB_INDEX_TYPE_UINT8) return __ldg((const uint8_t *)D.indices + k);
    return __ldg((const uint32_t *)D.indices + k);
}

// Index-buffer positions of triangle t of a (sub-)draw whose indices start at
// position base: setBatchIndices (Renderer.cpp:49-145).  Provoking vertex
// first: list (3t, 3t+1, 3t+2), strip (t, t+1+odd, t+2-odd), odd = t & 1, fan
// (t+1, t+2, 0); last: list (3t+2, 3t, 3t+1), strip (t+2, t+odd, t+1-odd), fan
// (t+2, 0, t+1).
__device__ __forceinline__ void tri_positions(const DrawParams &D, uint32_t base, uint32_t t, uint32_t &k0, uint32_t &k1, uint32_t &k2)
{
    const uint32_t odd = t & 1;
    if(D.topology == SWGB_TOPOLOGY_TRIANGLE_STRIP)
    {
        if(D.provokingLast) { k0 = t + 2; k1 = t + odd; k2 = t + 1 - odd; }
        else { k0 = t; k1 = t + 1 + odd; k2 = t + 2 - odd; }
    }
    else if(D.topology == SWGB_TOPOLOGY_TRIANGLE_FAN)
    {
        if(D.provokingLast) { k0 = t + 2; k1 = 0; k2 = t + 1; }
        else { k0 = t + 1; k1 = t + 2; k2 = 0; }
    }
    else
    {
        if(D.provokingLast) { k0 = 3 * t + 2; k1 = 3 * t; k2 = 3 * t + 1; }
        else { k0 = 3 * t; k1 = 3 * t + 1; k2 = 3 * t + 2; }
    }
    k0 += base;
    k1 += base;
    k2 += base;
}

// Primitive restart: slot p (an index position) is a triangle when it is not
// a restart index and completes one inside its segment -- the sub-draws
// vk::IndexBuffer::getIndexBuffers splits off (src/Device/Context.cpp:49-91),
// each drawn from its first index.  base = the segment's first position, t =
// the triangle's number inside it.
constexpr int RESTART_BLOCK = 1024;
__device__ __forceinline__ bool restart_slot(const DrawParams &D, uint32_t p, uint32_t &base, uint32_t &t)
{
    if(fetch_index(D, p) == D.restartValue) return false;
    base = max(__ldg(D.restartLocal + p), __ldg(D.restartCarry + p / RESTART_BLOCK));
    const uint32_t d = p - base;
    if(D.topology == SWGB_TOPOLOGY_TRIANGLE_LIST)
    {
        if(d % 3 != 2) return false;
        t = d / 3;
    }
    else
    {
        if(d < 2) return false;
        t = d - 2;
    }
    return true;
}

// Triangle slot t of the draw is a triangle (always, without primitive restart).
__device__ __forceinline__ bool tri_valid(const DrawParams &D, uint32_t t)
{
    uint32_t base, local;
    return !D.restart || restart_slot(D, t, base, local);
}

// Post-transform vertex slots of triangle slot t (valid, see tri_valid),
// through the index buffer of an indexed draw.
__device__ __forceinline__ void tri_slots(const DrawParams &D, uint32_t t, uint32_t &i0, uint32_t &i1, uint32_t &i2)
{
    uint32_t base = 0, local = t, k0, k1, k2;
    if(D.restart) restart_slot(D, t, base, local);
    tri_positions(D, base, local, k0, k1, k2);
    i0 = fetch_index(D, k0);
    i1 = fetch_index(D, k1);
    i2 = fetch_index(D, k2);
}

#ifndef SWGB_RASTER_TU
// Primitive restart, first pass: per block of RESTART_BLOCK index positions,
// the segment start of every position as far as the block sees it (one past
// the block's last restart index at or before it, else 0), and the block's
// last such value for the carry pass.
__global__ void __launch_bounds__(RESTART_BLOCK) k_restart_blocks(const __grid_constant__ DrawParams D, uint32_t *local, uint32_t *blockLast)
{
    __shared__ uint32_t warpMax[RESTART_BLOCK / 32];
    const uint32_t p = blockIdx.x * RESTART_BLOCK + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t v = (p < D.count && fetch_index(D, p) == D.restartValue) ? p + 1 : 0u;
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
    {
        const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if(lane >= o) v = max(v, u);
    }
    if(lane == 31) warpMax[warp] = v;
    __syncthreads();
    if(warp == 0)
    {
        uint32_t w = warpMax[lane];
#pragma unroll
        for(int o = 1; o < 32; o <<= 1)
        {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if(lane >= o) w = max(w, u);
        }
        warpMax[lane] = w;  // inclusive prefix max over the block's warps
    }
    __syncthreads();
    if(warp > 0) v = max(v, warpMax[warp - 1]);
    if(p < D.count) local[p] = v;
    if(threadIdx.x == RESTART_BLOCK - 1) blockLast[blockIdx.x] = v;
}

// Primitive restart, carry pass (one block): carry[b] = the largest segment
// start of the blocks before b, so a position's segment start is
// max(local[p], carry[p / RESTART_BLOCK]).
__global__ void __launch_bounds__(1024) k_restart_carry(const uint32_t *blockLast, uint32_t *carry, uint32_t nblocks)
{
    __shared__ uint32_t chunkMax;
    uint32_t run = 0;
    for(uint32_t c0 = 0; c0 < nblocks; c0 += blockDim.x)
    {
        const uint32_t b = c0 + threadIdx.x;
        uint32_t v = b < nblocks ? blockLast[b] : 0u;
        // exclusive prefix max inside the chunk, by warps then across warps
        __shared__ uint32_t wm[32];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t incl = v;
#pragma unroll
        for(int o = 1; o < 32; o <<= 1)
        {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if(lane >= o) incl = max(incl, u);
        }
        if(lane == 31) wm[warp] = incl;
        __syncthreads();
        if(warp == 0)
        {
            uint32_t w = wm[lane];
#pragma unroll
            for(int o = 1; o < 32; o <<= 1)
            {
                const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if(lane >= o) w = max(w, u);
            }
            wm[lane] = w;
        }
        __syncthreads();
        const uint32_t before = max(run, warp > 0 ? wm[warp - 1] : 0u);
        const uint32_t excl = max(before, __shfl_up_sync(0xFFFFFFFFu, incl, 1) * (lane > 0));
        if(b < nblocks) carry[b] = lane > 0 ? excl : before;
        if(threadIdx.x == blockDim.x - 1) chunkMax = max(before, incl);
        __syncthreads();
        run = chunkMax;
        __syncthreads();
    }
}
#endif  // SWGB_RASTER_TU

struct CVert { float x, y, z, w; };

__device__ __forceinline__ float plane_dist(const CVert &v, int plane)
{
    switch(plane)
    {
    case 0: return v.z;
    case 1: return v.w - v.z;
    case 2: return v.w + v.x;
    case 3: return v.w - v.x;
    case 4: return v.w - v.y;
    default: return v.w + v.y;
    }
}

// clipEdge (src/Device/Clipper.cpp:22-30)
__device__ __forceinline__ CVert clip_edge(const CVert &Vi, const CVert &Vj, float di, float dj)
{
    float D = 1.0f / (dj - di);
    CVert o;
    o.x = (dj * Vi.x - di * Vj.x) * D;
    o.y = (dj * Vi.y - di * Vj.y) * D;
    o.z = (dj * Vi.z - di * Vj.z) * D;
    o.w = (dj * Vi.w - di * Vj.w) * D;
    return o;
}

// Clipper::Clip (src/Device/Clipper.cpp:271-299): NEAR, FAR, LEFT, RIGHT,
// TOP, BOTTOM, each Sutherland-Hodgman pass as clipNear..clipBottom (:32-265).
static __device__ int clip_polygon(CVert *P, int n, int flagsOr)
{
    const int order[6] = {CLIP_NEAR, CLIP_FAR, CLIP_LEFT, CLIP_RIGHT, CLIP_TOP, CLIP_BOTTOM};
    CVert T[MAX_POLY];
    for(int k = 0; k < 6; k++)
    {
        if(n < 3) break;
        if(!(flagsOr & order[k])) continue;
        int t = 0;
        for(int i = 0; i < n; i++)
        {
            int j = i == n - 1 ? 0 : i + 1;
            float di = plane_dist(P[i], k);
            float dj = plane_dist(P[j], k);
            if(di >= 0.0f)
            {
                if(t < MAX_POLY) T[t] = P[i];
                t++;
                if(dj < 0.0f)
                {
                    if(t < MAX_POLY) T[t] = clip_edge(P[i], P[j], di, dj);
                    t++;
                }
            }
            else if(dj > 0.0f)
            {
                if(t < MAX_POLY) T[t] = clip_edge(P[j], P[i], dj, di);
                t++;
            }
        }
        n = t < MAX_POLY ? t : MAX_POLY;
        for(int i = 0; i < n; i++) P[i] = T[i];
    }
    return n;
}

// Span x of one polygon edge at row y (SetupRoutine::edge, src/Pipeline/SetupRoutine.cpp:550-621):
// the DDA value after (y - y1) steps, computed in closed form.  Returns false
// when the edge does not write row y.  *isRight tells which span it writes.
struct EdgeDDA {
    int32_t y1, yMin, yMax;  // rows written: [yMin, yMax)
    int32_t x, d, Q, R, D;   // state at row y1
    bool right;
};

__device__ __forceinline__ bool edge_setup(const DrawParams &D, int32_t Xa, int32_t Ya, int32_t Xb, int32_t Yb, EdgeDDA &e)
{
    if(Ya == Yb) return false;
    bool swap = Yb < Ya;
    int32_t X1 = swap ? Xb : Xa, X2 = swap ? Xa : Xb;
    int32_t Y1 = swap ? Yb : Ya, Y2 = swap ? Ya : Yb;
    int32_t y1 = (Y1 + 0xFF) >> 8;
    int32_t y2 = (Y2 + 0xFF) >> 8;
    e.y1 = y1;
    e.yMin = max(y1, D.sy0);
    e.yMax = min(y2, D.sy1);
    if(!(e.yMin < e.yMax)) return false;
    e.right = swap;
    int32_t DX12 = X2 - X1, DY12 = Y2 - Y1;
    int32_t FDX12 = (int32_t)((uint32_t)DX12 << 8), FDY12 = (int32_t)((uint32_t)DY12 << 8);
    int32_t X = (int32_t)((uint32_t)DX12 * (uint32_t)(((uint32_t)y1 << 8) - (uint32_t)Y1) + (uint32_t)(X1 & 0xFF) * (uint32_t)DY12);
    int32_t x = (X1 >> 8) + X / FDY12;
    int32_t d = X % FDY12;
    int32_t c = (-d) >> 31;
    x -= c;
    d -= c & FDY12;
    int32_t Q = FDX12 / FDY12, R = FDX12 % FDY12;
    int32_t fl = R >> 31;
    Q += fl;
    R += fl & FDY12;
    e.x = x; e.d = d; e.Q = Q; e.R = R; e.D = FDY12;
    return true;
}

// x of the edge at row y (y1 <= y): x_k = x0 + k*Q + ceil((d0 + k*R) / D),
// identical to k iterations of the reference's DDA step.
__device__ __forceinline__ int32_t edge_x_at(const EdgeDDA &e, int32_t y, int32_t *dOut)
{
    int32_t k = y - e.y1;
    if(k == 0)
    {
        if(dOut) *dOut = e.d;
        return e.x;
    }
    long long num = (long long)e.d + (long long)k * e.R;  // > -D
    long long m = num > 0 ? (num + e.D - 1) / e.D : 0;
    if(dOut) *dOut = (int32_t)(num - m * e.D);
    return (int32_t)((uint32_t)e.x + (uint32_t)k * (uint32_t)e.Q + (uint32_t)m);
}

__device__ __forceinline__ int32_t clamp_x(const DrawParams &D, int32_t x) { return min(max(x, D.sx0), D.sx1); }

// Span (left, right) of a polygon at row y: the last edge (in edge order)
// that writes the row wins, as in the reference's outline buffer.
static __device__ void span_at(const DrawParams &D, const int32_t *X, const int32_t *Y, int n, int dW, int32_t y, int32_t &l, int32_t &r)
{
    l = 0; r = 0;
    for(int i = 0; i < n; i++)
    {
        int ia = i + 1 - dW, ib = i + dW;
        ia = ia == n ? 0 : ia;
        ib = ib == n ? 0 : ib;
        EdgeDDA e;
        if(!edge_setup(D, X[ia], Y[ia], X[ib], Y[ib], e)) continue;
        if(y < e.yMin || y >= e.yMax) continue;
        int32_t x = clamp_x(D, edge_x_at(e, y, nullptr));
        if(e.right) r = x; else l = x;
    }
}

// Writes the spans of rows [yMin, yMax) of a polygon into sp[0 .. yMax-yMin)
// (left | right << 16), edge by edge in the reference's order, so that the
// last edge writing a row wins exactly as in the outline buffer
// (SetupRoutine.cpp:230-240,550-621).  Every row in the range is written by at
// least one edge per side: the polygon is closed.
static __device__ void write_spans(const DrawParams &D, const int32_t *X, const int32_t *Y, int n, int dW, int32_t yMin, uint32_t *sp)
{
    for(int i = 0; i < n; i++)
    {
        int ia = i + 1 - dW, ib = i + dW;
        ia = ia == n ? 0 : ia;
        ib = ib == n ? 0 : ib;
        EdgeDDA e;
        if(!edge_setup(D, X[ia], Y[ia], X[ib], Y[ib], e)) continue;
        int32_t dd;
        int32_t x = edge_x_at(e, e.yMin, &dd);
        uint16_t *h = reinterpret_cast<uint16_t *>(sp) + (e.right ? 1 : 0);
        for(int32_t y = e.yMin; y < e.yMax; y++)
        {
            h[2 * (y - yMin)] = (uint16_t)clamp_x(D, x);
            x += e.Q;
            dd += e.R;
            int32_t of = (-dd) >> 31;
            dd -= e.D & of;
            x -= of;
        }
    }
}

// One 256-triangle block of a draw (block index 'blk' within the draw).
constexpr int PLANE_V = 6;  // varying components with plane equations (colour + uv)
constexpr int PLANE_ZBIAS = 8 + 3 * PLANE_V;  // the triangle's depth bias (Primitive::zBias)
constexpr int PLANES = PLANE_ZBIAS + 1;
constexpr int PLANES_STORED = 28;  // PLANES rounded up to whole float4s


__device__ __forceinline__ float vary(const float4 &a, const float4 &b, int k)
{
    // varying k of a post-transform vertex: float4[2].yzw then float4[3].xyzw
    switch(k)
    {
    case 0: return a.y;
    case 1: return a.z;
    case 2: return a.w;
    case 3: return b.x;
    case 4: return b.y;
    case 5: return b.z;
    default: return b.w;
    }
}

// Plane equations of a triangle (SetupRoutine.cpp:270-548) from its three
// post-transform vertex records, v[k] = float4 k of the vertex (k = 0: clip
// position, 1: X, Y, flags, projected z, 2: rhw + varyings 0-2, 3: varyings
// 3-6): x0, y0 of the rotated first vertex, z (A, B, C), w (A, B, C) and each
// varying (A, B, C), PLANES floats, unused ones zero.  The setup stage
// evaluates them once per triangle; the raster stage loads them for every bin
// the triangle touches.
__device__ __forceinline__ float4 select3(int o, const float4 &a, const float4 &b, const float4 &c)
{
    return o == 0 ? a : (o == 1 ? b : c);
}

__device__ __forceinline__ void triangle_planes(const DrawParams &D, const float4 c[3], const float4 p[3], const float4 a[3],
                                                const float4 b[3], float pl[PLANES_STORED])
{
#pragma unroll
    for(int k = 0; k < PLANES_STORED; k++) pl[k] = 0.0f;
    // sort by minimum y, then maximum w (SetupRoutine.cpp:270-294)
    int o0 = 0, o1 = 1, o2 = 2, tt;
    {
        float ym = rmin(rmin(c[0].y, c[1].y), c[2].y);
        if(ym == c[1].y) { tt = o0; o0 = o1; o1 = o2; o2 = tt; }
        if(ym == c[2].y) { tt = o2; o2 = o1; o1 = o0; o0 = tt; }
    }
    const float cw0 = c[0].w, cw1 = c[1].w, cw2 = c[2].w;
    {
        float w0 = o0 == 0 ? cw0 : (o0 == 1 ? cw1 : cw2);
        float w1 = o1 == 0 ? cw0 : (o1 == 1 ? cw1 : cw2);
        float w2 = o2 == 0 ? cw0 : (o2 == 1 ? cw1 : cw2);
        float wm = rmax(rmax(w0, w1), w2);
        if(wm == w1) { tt = o0; o0 = o1; o1 = o2; o2 = tt; }
        if(wm == w2) { tt = o2; o2 = o1; o1 = o0; o0 = tt; }
    }
    const float w1 = o1 == 0 ? cw0 : (o1 == 1 ? cw1 : cw2);
    const float w2 = o2 == 0 ? cw0 : (o2 == 1 ? cw1 : cw2);
    const float4 P0 = select3(o0, p[0], p[1], p[2]), P1 = select3(o1, p[0], p[1], p[2]), P2 = select3(o2, p[0], p[1], p[2]);
    const float4 A0 = select3(o0, a[0], a[1], a[2]), A1 = select3(o1, a[0], a[1], a[2]), A2 = select3(o2, a[0], a[1], a[2]);
    const float rhw0 = A0.x;
    int32_t X0 = __float_as_int(P0.x), X1 = __float_as_int(P1.x), X2 = __float_as_int(P2.x);
    int32_t Y0 = __float_as_int(P0.y), Y1 = __float_as_int(P1.y), Y2 = __float_as_int(P2.y);
    const float inv = 1.0f / 256.0f;
    pl[0] = (float)X0 * inv;
    pl[1] = (float)Y0 * inv;
    X1 -= X0; Y1 -= Y0; X2 -= X0; Y2 -= Y0;
    float x1 = (w1 * inv) * (float)X1, y1 = (w1 * inv) * (float)Y1;
    float x2 = (w2 * inv) * (float)X2, y2 = (w2 * inv) * (float)Y2;
    float ar = x1 * y2 - x2 * y1;
    float M0x = 0.0f, M0y = 0.0f, M1x = 0.0f, M1y = 0.0f, M2x = 0.0f, M2y = 0.0f;
    const float M0z = rhw0, M1z = 0.0f, M2z = 0.0f;
    if(ar != 0.0f)
    {
        float A = 1.0f / ar;
        float Dd = A * rhw0;
        M0x = (y1 * w2 - y2 * w1) * Dd;
        M0y = (x2 * w1 - x1 * w2) * Dd;
        M1x = y2 * A;
        M1y = (-x2) * A;
        M2x = (-y1) * A;
        M2y = x1 * A;
    }
    pl[5] = (M0x + M1x) + M2x;
    pl[6] = (M0y + M1y) + M2y;
    pl[7] = (M0z + M1z) + M2z;
    if(D.depthTest)
    {
        float z0 = P0.w, z1 = P1.w - z0, z2 = P2.w - z0;
        float fx1 = (float)X1 * inv, fy1 = (float)Y1 * inv;
        float fx2 = (float)X2 * inv, fy2 = (float)Y2 * inv;
        float Dz = D.depthRange / (fx1 * fy2 - fx2 * fy1);
        pl[2] = (fy2 * z1 - fy1 * z2) * Dz;
        pl[3] = (fx1 * z2 - fx2 * z1) * Dz;
        pl[4] = z0 * D.depthRange + D.depthNear;
        // depth bias (SetupRoutine.cpp:417-476)
        if(D.biasConstant != 0.0f || D.biasSlope != 0.0f)
        {
            float bias = 0.0f;
            if(D.biasConstant != 0.0f)
            {
                float r;  // minimum resolvable difference
                if(D.depth16) r = 1.01f / 0xFFFF;
                else
                {
                    // 2^(e - 23), e the largest exponent of the depths; the
                    // reference forms Z1, Z2 from the vertex differences
                    const float Z0 = pl[4], Z1 = z1 * D.depthRange + D.depthNear, Z2 = z2 * D.depthRange + D.depthNear;
                    const int e = max(max(__float_as_int(Z0) & 0x7F800000, __float_as_int(Z1) & 0x7F800000),
                                      __float_as_int(Z2) & 0x7F800000);
                    r = __int_as_float(e) * (1.0f / (1 << 23));
                }
                bias = r * D.biasConstant;
            }
            if(D.biasSlope != 0.0f) bias += rmax(fabsf(pl[2]), fabsf(pl[3])) * D.biasSlope;
            if(D.biasClamp != 0.0f) bias = D.biasClamp > 0.0f ? rmin(bias, D.biasClamp) : rmax(bias, D.biasClamp);
            pl[PLANE_ZBIAS] = bias;
        }
    }
    const float4 B0 = select3(o0, b[0], b[1], b[2]), B1 = select3(o1, b[0], b[1], b[2]), B2 = select3(o2, b[0], b[1], b[2]);
#pragma unroll
    for(int k = 0; k < PLANE_V; k++)
    {
        if(k >= D.nv) break;
        float v0 = vary(A0, B0, k), v1 = vary(A1, B1, k), v2 = vary(A2, B2, k);
        pl[8 + 3 * k + 0] = (v0 * M0x + v1 * M1x) + v2 * M2x;
        pl[8 + 3 * k + 1] = (v0 * M0y + v1 * M1y) + v2 * M2y;
        pl[8 + 3 * k + 2] = (v0 * M0z + v1 * M1z) + v2 * M2z;
    }
}

// Clipped triangle (rare; out of line, its polygon arrays live in local
// memory): Clipper::Clip, the reprojection of the clipped polygon
// (SetupRoutine.cpp:125-145), its y range (:147-186) and x extent; a visible
// polygon is stored in the draw's polygon scratch for the span stage and the
// raster's edge walk.  Returns the vertex count (0: clipped away or empty y
// range; -1: polygon scratch full).
static __device__ __noinline__ int setup_clipped(const DrawParams &D, const float4 c0, const float4 c1, const float4 c2, int flagsOr,
                                                 int32_t &yMin, int32_t &yMax, int32_t &xMinS, int32_t &xMaxS, uint32_t &slot)
{
    CVert P[MAX_POLY];
    P[0] = {c0.x, c0.y, c0.z, c0.w};
    P[1] = {c1.x, c1.y, c1.z, c1.w};
    P[2] = {c2.x, c2.y, c2.z, c2.w};
    const int n = clip_polygon(P, 3, flagsOr);
    if(n < 3) return 0;
    int32_t X[MAX_POLY], Y[MAX_POLY];
    for(int i = 0; i < n; i++)
    {
        float w = P[i].w;
        float rhw = w != 0.0f ? 1.0f / w : 1.0f;
        X[i] = round_int(D.X0xF + (P[i].x * rhw) * D.WxF);
        Y[i] = round_int(D.Y0xF + (P[i].y * rhw) * D.HxF);
    }
    yMin = Y[0]; yMax = Y[0]; xMinS = X[0]; xMaxS = X[0];
    for(int i = 1; i < n; i++)
    {
        yMin = min(yMin, Y[i]); yMax = max(yMax, Y[i]);
        xMinS = min(xMinS, X[i]); xMaxS = max(xMaxS, X[i]);
    }
    if(D.ms > 1)
    {
        yMin = max((yMin + Y_MIN_MS_OFFSET) >> 8, D.sy0);
        yMax = min((yMax + Y_MAX_MS_OFFSET) >> 8, D.sy1);
    }
    else
    {
        yMin = max((yMin + 0xFF) >> 8, D.sy0);
        yMax = min((yMax + 0xFF) >> 8, D.sy1);
    }
    if(yMin >= yMax) return 0;
    slot = atomicAdd(D.polyCount, 1u);
    if(slot >= D.polyCapacity)
    {
        atomicOr(D.error, ERR_POLY_OVERFLOW);
        return -1;
    }
    for(int i = 0; i < n; i++) D.poly[(size_t)slot * MAX_POLY + i] = make_int2(X[i], Y[i]);
    return n;
}

// Span rows of a stored clipped polygon (write_spans per sample, rows
// [yMin, yMax)), and for one sample the trimmed range (SetupRoutine.cpp:243-264).
static __device__ __noinline__ void spans_clipped(const DrawParams &D, uint32_t slot, int n, int dW, int32_t yMin, int32_t yMax,
                                                  uint32_t *sp, int32_t &tMin, int32_t &tMax)
{
    int32_t X[MAX_POLY], Y[MAX_POLY];
    for(int i = 0; i < n; i++)
    {
        const int2 q = D.poly[(size_t)slot * MAX_POLY + i];
        X[i] = q.x; Y[i] = q.y;
    }
    const uint32_t rows = (uint32_t)(yMax - yMin);
    tMin = yMin;
    tMax = yMax;
    if(D.ms > 1)
    {
        // one outline per sample, the polygon shifted by -Xf/-Yf; rows no edge
        // writes stay empty and nothing is trimmed (SetupRoutine.cpp:188-240)
        for(int q = 0; q < 4; q++)
        {
            uint32_t *s = sp + (uint64_t)q * rows;
            for(uint32_t r = 0; r < rows; r++) s[r] = 0u;
            int32_t Xq[MAX_POLY], Yq[MAX_POLY];
            for(int i = 0; i < n; i++) { Xq[i] = X[i] - XF[q]; Yq[i] = Y[i] - YF[q]; }
            write_spans(D, Xq, Yq, n, dW, yMin, s);
        }
        return;
    }
    write_spans(D, X, Y, n, dW, yMin, sp);
    while(tMin < tMax)
    {
        const uint32_t s = sp[tMin - yMin];
        if((s & 0xFFFFu) != (s >> 16)) break;
        tMin++;
    }
    while(tMax > tMin)
    {
        const uint32_t s = sp[tMax - 1 - yMin];
        if((s & 0xFFFFu) != (s >> 16)) break;
        tMax--;
    }
}

// Trimmed y range of a clipped polygon whose rows did not fit the span
// scratch, by direct evaluation (k_raster then walks its edges itself).
static __device__ __noinline__ void trim_clipped_unstored(const DrawParams &D, uint32_t slot, int n, int dW, int32_t &yMin, int32_t &yMax)
{
    int32_t X[MAX_POLY], Y[MAX_POLY];
    for(int i = 0; i < n; i++)
    {
        const int2 q = D.poly[(size_t)slot * MAX_POLY + i];
        X[i] = q.x; Y[i] = q.y;
    }
    int32_t l, r;
    while(yMin < yMax)
    {
        span_at(D, X, Y, n, dW, yMin, l, r);
        if(l != r) break;
        yMin++;
    }
    while(yMax > yMin)
    {
        span_at(D, X, Y, n, dW, yMax - 1, l, r);
        if(l != r) break;
        yMax--;
    }
}

// Span rows [yMin, yMax) of an N-vertex outline in registers -- an unclipped
// triangle (shifted by the sample offset for 4x MSAA) or a clipped polygon of
// at most 4 vertices -- row by row: each row's left and right come from the
// edges covering it, walked by the reference's DDA (SetupRoutine::edge,
// :550-621), and are stored as one word.  The edges on one side of a convex
// outline cover disjoint rows, so this equals the reference's edge-by-edge
// outline.  Rows no edge covers get the empty span 0 (only sample outlines of
// 4x MSAA have them).  Returns the first and one past the last row with
// left != right (the trim of :243-264; first = last = yMax when every row is
// empty).
template<int N>
__device__ __forceinline__ void spans_outline(const DrawParams &D, const int32_t (&Xs)[N], const int32_t (&Ys)[N], int dW, int32_t yMin,
                                              int32_t yMax, uint32_t *sp, int32_t &first, int32_t &last)
{
    // edges in the reference's order: edge i runs from vertex i+1-d to vertex i+d
    EdgeDDA e[N];
    bool ok[N];
    int32_t ex[N], ed[N], y0[N];
    uint32_t nr[N];
#pragma unroll
    for(int i = 0; i < N; i++)
    {
        int ia = i + 1 - dW, ib = i + dW;
        ia = ia == N ? 0 : ia;
        ib = ib == N ? 0 : ib;
        ok[i] = edge_setup(D, Xs[ia], Ys[ia], Xs[ib], Ys[ib], e[i]);
        ex[i] = 0;
        ed[i] = 0;
        if(ok[i]) ex[i] = edge_x_at(e[i], e[i].yMin, &ed[i]);
        // rows of the edge as one unsigned range test: y - yMin < rows (none
        // for an edge that writes no row)
        y0[i] = ok[i] ? e[i].yMin : 0;
        nr[i] = ok[i] ? (uint32_t)(e[i].yMax - e[i].yMin) : 0u;
    }
    first = yMax;
    last = yMax;
    int32_t lastNonEmpty = yMin - 1;
    for(int32_t y = yMin; y < yMax; y++)
    {
        int32_t l = 0, r = 0;
#pragma unroll
        for(int i = 0; i < N; i++)
        {
            if((uint32_t)(y - y0[i]) < nr[i])
            {
                const int32_t x = clamp_x(D, ex[i]);
                if(e[i].right) r = x; else l = x;
                ex[i] += e[i].Q;
                ed[i] += e[i].R;
                const int32_t of = (-ed[i]) >> 31;
                ed[i] -= e[i].D & of;
                ex[i] -= of;
            }
        }
        sp[y - yMin] = (uint32_t)(l & 0xFFFF) | ((uint32_t)r << 16);
        if(l != r)
        {
            if(first == yMax) first = y;
            lastNonEmpty = y;
        }
    }
    if(first < yMax) last = lastNonEmpty + 1;
}

__device__ __forceinline__ void spans_triangle(const DrawParams &D, int32_t X0, int32_t Y0, int32_t X1, int32_t Y1, int32_t X2,
                                               int32_t Y2, int dW, int32_t yMin, int32_t yMax, uint32_t *sp, int32_t &first,
                                               int32_t &last)
{
    const int32_t Xs[3] = {X0, X1, X2}, Ys[3] = {Y0, Y1, Y2};
    spans_outline<3>(D, Xs, Ys, dW, yMin, yMax, sp, first, last);
}

// Clipped triangle whose vertices lie outside one clip plane only (plane k of
// Clipper::Clip's order): that plane's Sutherland-Hodgman pass (clipNear ..
// clipBottom, src/Device/Clipper.cpp:32-265) on the three vertices in
// registers -- each vertex i emits itself when inside and the crossing of
// edge (i, i+1) when the edge crosses, in the pass's order -- then the
// reprojection, y range and x extent as setup_clipped.  The polygon (at most
// 4 vertices, X/Y) stays in registers for the span rows and is also stored
// in the polygon scratch for the raster's fallback.  Returns the vertex count
// (0: clipped away or empty y range; -1: polygon scratch full).
static __device__ __forceinline__ int setup_clipped_one(const DrawParams &D, const float4 c0, const float4 c1, const float4 c2, int k,
                                                        int32_t &yMin, int32_t &yMax, int32_t &xMinS, int32_t &xMaxS, uint32_t &slot,
                                                        int32_t (&X)[4], int32_t (&Y)[4])
{
    const CVert P[3] = {{c0.x, c0.y, c0.z, c0.w}, {c1.x, c1.y, c1.z, c1.w}, {c2.x, c2.y, c2.z, c2.w}};
    float d[3];
#pragma unroll
    for(int i = 0; i < 3; i++) d[i] = plane_dist(P[i], k);
    // emitted vertices in order: P_i when inside, then E_i when edge (i, i+1) crosses
    bool inP[3], inE[3];
    CVert E[3];
    int posP[3], posE[3], t = 0;
#pragma unroll
    for(int i = 0; i < 3; i++)
    {
        const int j = i == 2 ? 0 : i + 1;
        inP[i] = d[i] >= 0.0f;
        inE[i] = inP[i] ? d[j] < 0.0f : d[j] > 0.0f;
        E[i] = inP[i] ? clip_edge(P[i], P[j], d[i], d[j]) : clip_edge(P[j], P[i], d[j], d[i]);
        posP[i] = t;
        t += inP[i] ? 1 : 0;
        posE[i] = t;
        t += inE[i] ? 1 : 0;
    }
    const int n = t;
    if(n < 3) return 0;
#pragma unroll
    for(int m = 0; m < 4; m++)
    {
        CVert v = P[0];
#pragma unroll
        for(int i = 0; i < 3; i++)
        {
            if(inP[i] && posP[i] == m) v = P[i];
            if(inE[i] && posE[i] == m) v = E[i];
        }
        const float rhw = v.w != 0.0f ? 1.0f / v.w : 1.0f;
        X[m] = round_int(D.X0xF + (v.x * rhw) * D.WxF);
        Y[m] = round_int(D.Y0xF + (v.y * rhw) * D.HxF);
    }
    if(n == 3)
    {
        X[3] = X[2];
        Y[3] = Y[2];
    }
    yMin = min(min(Y[0], Y[1]), min(Y[2], Y[3]));
    yMax = max(max(Y[0], Y[1]), max(Y[2], Y[3]));
    xMinS = min(min(X[0], X[1]), min(X[2], X[3]));
    xMaxS = max(max(X[0], X[1]), max(X[2], X[3]));
    yMin = max((yMin + 0xFF) >> 8, D.sy0);
    yMax = min((yMax + 0xFF) >> 8, D.sy1);
    if(yMin >= yMax) return 0;
    slot = atomicAdd(D.polyCount, 1u);
    if(slot >= D.polyCapacity)
    {
        atomicOr(D.error, ERR_POLY_OVERFLOW);
        return -1;
    }
#pragma unroll
    for(int m = 0; m < 4; m++)
        if(m < n) D.poly[(size_t)slot * MAX_POLY + m] = make_int2(X[m], Y[m]);
    return n;
}

// One SETUP_THREADS-triangle block of a draw (block index 'blk' within the
// draw), one thread per triangle: trivial reject, culling, clipping, y range,
// span rows (allocated per warp), pixel box, record and plane equations; per
// warp the chunk box, the super-chunk box and the counters.  No block barrier.
// CLIP_ONE: triangles clipped by one plane take setup_clipped_one (the
// batched kernel, whose draw records live in global memory, leaves it out:
// it would spill there).
template<bool CLIP_ONE>
__device__ __forceinline__ void setup_body(const DrawParams &D, uint32_t blk)
{
    const uint32_t t = blk * SETUP_THREADS + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    short4 box = make_short4(0, 0, 0, 0);
    TriInfo inf = {0u, 0u, 0u, 0u};
    int cntIn = 0, cntClip = 0, cntVis = 0;
    bool cand = false;
    int n = 3, dW = 1, frontBit = 0;
    int32_t X0 = 0, X1 = 0, X2 = 0, Y0 = 0, Y1 = 0, Y2 = 0;
    int32_t yMin = 0, yMax = 0, xMinS = 0, xMaxS = 0;
    uint32_t slot = 0, vs0 = 0, vs1 = 0, vs2 = 0;  // post-transform vertex slots
    int32_t X3 = 0, Y3 = 0;  // fourth vertex of a polygon clipped by one plane
    bool clipOne = false;    // the polygon (X0..X3, Y0..Y3) came from setup_clipped_one
    float area2 = 0.0f;      // |doubled area| of the snapped triangle, 1/256-pixel units squared
    if(t < D.count && tri_valid(D, t))
    {
        cntIn = 1;
        tri_slots(D, t, vs0, vs1, vs2);
        bool ok = true;
        if(D.indexType != SWGB_INDEX_TYPE_NONE && (vs0 >= D.vertexCount || vs1 >= D.vertexCount || vs2 >= D.vertexCount))
        {
            atomicOr(D.error, ERR_INDEX_RANGE);
            ok = false;
        }
        if(ok)
        {
            float4 vp[3], vc[3];
            vp[0] = D.ptv[(size_t)vs0 * 4 + 1]; vp[1] = D.ptv[(size_t)vs1 * 4 + 1]; vp[2] = D.ptv[(size_t)vs2 * 4 + 1];
            vc[0] = D.ptv[(size_t)vs0 * 4]; vc[1] = D.ptv[(size_t)vs1 * 4]; vc[2] = D.ptv[(size_t)vs2 * 4];
            const int f0 = __float_as_int(vp[0].z), f1 = __float_as_int(vp[1].z), f2 = __float_as_int(vp[2].z);
            X0 = __float_as_int(vp[0].x); X1 = __float_as_int(vp[1].x); X2 = __float_as_int(vp[2].x);
            Y0 = __float_as_int(vp[0].y); Y1 = __float_as_int(vp[1].y); Y2 = __float_as_int(vp[2].y);
            // setupSolidTriangles trivial reject (src/Device/Renderer.cpp:749-765)
            if((f0 & f1 & f2) == CLIP_FINITE)
            {
                const int flagsOr = f0 | f1 | f2;
                cntClip = flagsOr != CLIP_FINITE;  // the triangle goes through the clipper (Renderer.cpp:758-765)
                // Culling (SetupRoutine.cpp:73-120) on the triangle's own snapped
                // vertices; it rejects a triangle the same whether or not the
                // clipper ran first.
                float x0 = (float)X0, x1 = (float)X1, x2 = (float)X2;
                float y0 = (float)Y0, y1 = (float)Y1, y2 = (float)Y2;
                float A = ((y0 - y2) * x1 + (y2 - y1) * x0) + (y1 - y0) * x2;
                int32_t w0w1w2 = __float_as_int(vc[0].w) ^ __float_as_int(vc[1].w) ^ __float_as_int(vc[2].w);
                if(w0w1w2 < 0) A = -A;
                area2 = fabsf(A);
                bool front = D.frontFace == SWGB_FRONT_FACE_COUNTER_CLOCKWISE ? (A >= 0.0f) : (A <= 0.0f);
                frontBit = front ? 1 : 0;
                bool keep = !((D.cullMode & SWGB_CULL_FRONT) && front) && !((D.cullMode & SWGB_CULL_BACK) && !front);
                dW = A > 0.0f ? 1 : 0;
                const int planes = flagsOr & CLIP_FRUSTUM;
                if(CLIP_ONE && keep && cntClip && D.ms == 1 && (planes & (planes - 1)) == 0)
                {
                    // one plane (the common case: triangles across a side of the
                    // view): the clipper's single pass in registers
                    const int k = planes == CLIP_NEAR ? 0 : planes == CLIP_FAR ? 1 : planes == CLIP_LEFT ? 2 :
                                  planes == CLIP_RIGHT ? 3 : planes == CLIP_TOP ? 4 : 5;
                    int32_t PX[4], PY[4];
                    n = setup_clipped_one(D, vc[0], vc[1], vc[2], k, yMin, yMax, xMinS, xMaxS, slot, PX, PY);
                    cand = n >= 3;
                    clipOne = true;
                    X0 = PX[0]; X1 = PX[1]; X2 = PX[2]; X3 = PX[3];
                    Y0 = PY[0]; Y1 = PY[1]; Y2 = PY[2]; Y3 = PY[3];
                }
                else if(keep && cntClip)
                {
                    // through temporaries: a local whose address reaches an
                    // out-of-line call lives in local memory on every path
                    int32_t a0 = yMin, a1 = yMax, a2 = xMinS, a3 = xMaxS;
                    uint32_t a4 = slot;
                    n = setup_clipped(D, vc[0], vc[1], vc[2], flagsOr, a0, a1, a2, a3, a4);
                    yMin = a0; yMax = a1; xMinS = a2; xMaxS = a3; slot = a4;
                    cand = n >= 3;
                }
                else if(keep)
                {
                    yMin = min(min(Y0, Y1), Y2); yMax = max(max(Y0, Y1), Y2);
                    xMinS = min(min(X0, X1), X2); xMaxS = max(max(X0, X1), X2);
                    // Vertical range (SetupRoutine.cpp:147-186)
                    if(D.ms > 1)
                    {
                        yMin = max((yMin + Y_MIN_MS_OFFSET) >> 8, D.sy0);
                        yMax = min((yMax + Y_MAX_MS_OFFSET) >> 8, D.sy1);
                    }
                    else
                    {
                        yMin = max((yMin + 0xFF) >> 8, D.sy0);
                        yMax = min((yMax + 0xFF) >> 8, D.sy1);
                    }
                    cand = yMin < yMax;
                }
            }
        }
    }

    // ---- allocate span rows: warp scan + one atomic per warp -------------
    const uint32_t rows = cand ? (uint32_t)(yMax - yMin) : 0u;
    uint32_t incl = rows * (uint32_t)D.ms;
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
    {
        uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if(lane >= o) incl += u;
    }
    unsigned long long warpBase = 0ull;
    if(lane == 31 && incl) warpBase = atomicAdd(D.spanCount, (unsigned long long)incl);
    warpBase = __shfl_sync(0xFFFFFFFFu, warpBase, 31);
    const uint64_t off = (uint64_t)warpBase + (incl - rows * (uint32_t)D.ms);

    // a warp holding a 4-vertex polygon clipped by one plane writes every
    // outline of its lanes with the 4-edge writer in one pass: a triangle is the
    // 4-vertex outline with its last vertex repeated (the repeated vertex makes
    // an edge of zero height, which writes no row)
    const bool quad = cand && clipOne && n == 4;
    const bool warpQuad = __any_sync(0xFFFFFFFFu, quad);
    bool stored = false;
    if(cand)
    {
        stored = off + (uint64_t)rows * (uint32_t)D.ms <= (uint64_t)D.spanCapacity;
        uint32_t *sp = D.spans + off;
        int32_t tMin = yMin, tMax = yMax;
        if(stored && warpQuad && (!cntClip || clipOne) && D.ms == 1)
        {
            const int32_t Xs[4] = {X0, X1, X2, quad ? X3 : X2}, Ys[4] = {Y0, Y1, Y2, quad ? Y3 : Y2};
            spans_outline<4>(D, Xs, Ys, dW, yMin, yMax, sp, tMin, tMax);
        }
        else if(stored && cntClip && !clipOne)
        {
            int32_t a0 = tMin, a1 = tMax;  // temporaries, as above
            spans_clipped(D, slot, n, dW, yMin, yMax, sp, a0, a1);
            tMin = a0; tMax = a1;
        }
        else if(stored && D.ms > 1)
        {
            for(int q = 0; q < 4; q++)
            {
                int32_t f, l;
                spans_triangle(D, X0 - XF[q], Y0 - YF[q], X1 - XF[q], Y1 - YF[q], X2 - XF[q], Y2 - YF[q], dW, yMin, yMax,
                               sp + (uint64_t)q * rows, f, l);
            }
        }
        else if(stored)
            spans_triangle(D, X0, Y0, X1, Y1, X2, Y2, dW, yMin, yMax, sp, tMin, tMax);
        else if(D.ms > 1)
        {
            // span scratch full, 4x MSAA: nothing is trimmed (SetupRoutine.cpp:243);
            // k_raster walks the edges itself for this triangle
        }
        else if(cntClip)
        {
            int32_t a0 = tMin, a1 = tMax;
            trim_clipped_unstored(D, slot, n, dW, a0, a1);
            tMin = a0; tMax = a1;
        }
        else
        {
            // span scratch full: trim by direct evaluation; k_raster walks the
            // edges itself for this triangle
            const int32_t Xs[3] = {X0, X1, X2}, Ys[3] = {Y0, Y1, Y2};
            int32_t l, r;
            while(tMin < tMax)
            {
                span_at(D, Xs, Ys, 3, dW, tMin, l, r);
                if(l != r) break;
                tMin++;
            }
            while(tMax > tMin)
            {
                span_at(D, Xs, Ys, 3, dW, tMax - 1, l, r);
                if(l != r) break;
                tMax--;
            }
        }
        if(stored)
        {
            inf.spanOff = (uint32_t)(off + (uint64_t)(tMin - yMin));  // MSAA: tMin = yMin
            inf.rows = rows;
        }
        yMin = tMin;
        yMax = tMax;
    }
    if(cand && yMin < yMax)
    {
        // pixel box: covered x satisfy ceil(Xmin/256) <= left <= x < right <= ceil(Xmax/256)
        const int32_t pad = D.ms > 1 ? 96 : 0;  // farthest sample offset (Xf)
        int32_t bx0 = max(D.sx0, (xMinS - pad + 0xFF) >> 8);
        int32_t bx1 = max(bx0, min(D.sx1, (xMaxS + pad + 0xFF) >> 8));
        cntVis = 1;
        box = make_short4((short)bx0, (short)yMin, (short)bx1, (short)yMax);
        inf.info = (uint32_t)n | ((uint32_t)dW << 5) | ((uint32_t)cntClip << 6) | ((uint32_t)stored << 7) | ((uint32_t)frontBit << 8);
        if(!stored) inf.rows = 0;
        if(cntClip) inf.slot = slot;
    }
    D.triBox[t] = box;  // capacity is a whole number of setup blocks
    D.triInfo[t] = inf;
    if(cntVis)
    {
        // the vertex records again (cached): kept out of registers across the span loop
        float4 vc[3], vp[3], va[3], vb[3] = {make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
        vc[0] = D.ptv[(size_t)vs0 * 4]; vc[1] = D.ptv[(size_t)vs1 * 4]; vc[2] = D.ptv[(size_t)vs2 * 4];
        vp[0] = D.ptv[(size_t)vs0 * 4 + 1]; vp[1] = D.ptv[(size_t)vs1 * 4 + 1]; vp[2] = D.ptv[(size_t)vs2 * 4 + 1];
        va[0] = D.ptv[(size_t)vs0 * 4 + 2]; va[1] = D.ptv[(size_t)vs1 * 4 + 2]; va[2] = D.ptv[(size_t)vs2 * 4 + 2];
        if(D.nv > 3)
        {
            vb[0] = D.ptv[(size_t)vs0 * 4 + 3]; vb[1] = D.ptv[(size_t)vs1 * 4 + 3]; vb[2] = D.ptv[(size_t)vs2 * 4 + 3];
        }
        float pl[PLANES_STORED];
        triangle_planes(D, vc, vp, va, vb, pl);
        float4 *dst = D.planes + (size_t)t * (PLANES_STORED / 4);
#pragma unroll
        for(int k = 0; k < PLANES_STORED / 4; k++)
            if(k < D.planeVec4) dst[k] = make_float4(pl[4 * k], pl[4 * k + 1], pl[4 * k + 2], pl[4 * k + 3]);
    }
    if(D.binDiff)
    {
        // triangles per bin, for the raster's heaviest-first bin order: the
        // box's bin rectangle into a 2D difference array (k_bin_order
        // integrates).  Neighbouring triangles share corners, so lanes adding
        // to the same corner are merged first: one atomic per distinct corner.
        const bool hasBox = box.x < box.z && box.y < box.w;
        const unsigned act = __ballot_sync(0xFFFFFFFFu, hasBox);
        if(hasBox)
        {
            const int W = D.binsX + 1;
            const int xa = (box.x - D.binX0) / D.binW, xb = (box.z - 1 - D.binX0) / D.binW + 1;
            const int ya = (box.y - D.binY0) / D.binH, yb = (box.w - 1 - D.binY0) / D.binH + 1;
#pragma unroll
            for(int c = 0; c < 4; c++)
            {
                // corners (xa, ya) +1, (xb, ya) -1, (xa, yb) -1, (xb, yb) +1
                const int idx = (c < 2 ? ya : yb) * W + ((c == 0 || c == 2) ? xa : xb);
                const unsigned peers = __match_any_sync(act, idx);
                const int n = __popc(peers);
                if(lane == __ffs(peers) - 1) atomicAdd(&D.binDiff[idx], (c == 0 || c == 3) ? n : -n);
            }
        }
    }

    // ---- per warp: chunk box (CHUNK = 32 triangles), super-chunk box, counters ----
    const bool has = cntVis != 0;
    int bx0 = has ? box.x : 0x7FFF, by0 = has ? box.y : 0x7FFF;
    int bx1 = has ? box.z : -0x8000, by1 = has ? box.w : -0x8000;
    bx0 = __reduce_min_sync(0xFFFFFFFFu, bx0);
    by0 = __reduce_min_sync(0xFFFFFFFFu, by0);
    bx1 = __reduce_max_sync(0xFFFFFFFFu, bx1);
    by1 = __reduce_max_sync(0xFFFFFFFFu, by1);
    const int cntRej = __reduce_add_sync(0xFFFFFFFFu, cntIn - cntVis);
    cntIn = __reduce_add_sync(0xFFFFFFFFu, cntIn);
    cntClip = __reduce_add_sync(0xFFFFFFFFu, cntClip);
    cntVis = __reduce_add_sync(0xFFFFFFFFu, cntVis);
    static_assert(CHUNK == 32, "one chunk box per warp");
    const uint32_t chunk = blk * (SETUP_THREADS / CHUNK) + (uint32_t)warp;
    if(D.binCost && bx0 < bx1)
    {
        // the chunk's triangle area (each triangle's capped by its box) spread
        // evenly over the bins of the chunk box: a cost estimate for the bin
        // order, one difference-array update per corner
        uint32_t a = 0u;
        if(cntVis)
        {
            const uint32_t boxPx = (uint32_t)(box.z - box.x) * (uint32_t)(box.w - box.y);
            a = min((uint32_t)(area2 * (0.5f / 65536.0f)), boxPx);
        }
        a = __reduce_add_sync(0xFFFFFFFFu, a);
        const int W = D.binsX + 1;
        const int xa = (bx0 - D.binX0) / D.binW, xb = (bx1 - 1 - D.binX0) / D.binW + 1;
        const int ya = (by0 - D.binY0) / D.binH, yb = (by1 - 1 - D.binY0) / D.binH + 1;
        const uint32_t w = a / (uint32_t)((xb - xa) * (yb - ya));
        if(w && lane < 4)
        {
            const int idx = (lane < 2 ? ya : yb) * W + ((lane == 0 || lane == 2) ? xa : xb);
            atomicAdd(&D.binCost[idx], (lane == 0 || lane == 3) ? w : 0u - w);
        }
    }
    if(D.binFirst && bx0 < bx1)
    {
        // first chunk reaching each bin, for the order's tie-break; a chunk
        // spread over more than 256 bins leaves them to smaller chunks
        const int xa = (bx0 - D.binX0) / D.binW, xb = (bx1 - 1 - D.binX0) / D.binW;
        const int ya = (by0 - D.binY0) / D.binH, yb = (by1 - 1 - D.binY0) / D.binH;
        const int w = xb - xa + 1, area = w * (yb - ya + 1);
        if(area <= 256)
            for(int i = lane; i < area; i += 32) atomicMin(&D.binFirst[(ya + i / w) * D.binsX + xa + i % w], (int)chunk);
    }
    if(lane == 0)
    {
        D.chunkBox[chunk] = make_short4((short)bx0, (short)by0, (short)bx1, (short)by1);
        if(bx0 < bx1)
        {
            int4 *sb = D.superBox + chunk / SUPER;
            atomicMin(&sb->x, bx0);
            atomicMin(&sb->y, by0);
            atomicMax(&sb->z, bx1);
            atomicMax(&sb->w, by1);
        }
        if(cntIn) atomicAdd(&D.counters[0], (unsigned long long)cntIn);
        if(cntRej) atomicAdd(&D.counters[1], (unsigned long long)cntRej);
        if(cntClip) atomicAdd(&D.counters[2], (unsigned long long)cntClip);
        if(cntVis) atomicAdd(&D.counters[3], (unsigned long long)cntVis);
    }
}

#ifndef SWGB_RASTER_TU
__global__ void __launch_bounds__(SETUP_THREADS) k_setup(const __grid_constant__ DrawParams D) { setup_body<true>(D, blockIdx.x); }

// Order of a draw's bins for the persistent raster warps.  Longest first, by
// an estimated cost: the setup stage's two difference arrays integrated in
// shared memory into triangles per bin and spread triangle area per bin, the
// cost = area + triangles x (the draw's area per triangle), bucketed in
// eighth-octave steps, heaviest bucket first, so no heavy bin starts last and
// holds the frame's tail.  A bin's raster time follows its shaded fragments
// more than its triangle count (on the 1M-triangle 1080p height field,
// triangles + passed fragments explain 96% of the variance of the per-bin
// times, triangles alone 45%); the area is the part of that known before the
// raster.  Inside a bucket, bins reached earliest in the draw's triangle order
// go first (16 sub-buckets of the first chunk index), which reads the setup
// stage's oldest output first.  Measured on that frame: k_raster 0.896 ms with
// bit-length buckets of the triangle count (warps then finished between 0.76
// and 0.93 ms of the instrumented kernel: heavy bins started late), 0.833 ms
// with the cost; earlier, with count buckets, an arbitrary order inside the
// buckets had cost 4% against the first-touch one.  One block; bins with the
// same key are independent.
constexpr int BIN_ORDER_THREADS = 1024;
constexpr int BIN_ORDER_SUB = 16;
constexpr int BIN_ORDER_FINE = 33 * 8;  // eighth-octave steps of a 32-bit cost
constexpr int BIN_ORDER_KEYS = BIN_ORDER_FINE * BIN_ORDER_SUB;
__device__ __forceinline__ int bin_order_key(uint32_t cost, int first, int nchunks)
{
    const int len = cost > 0u ? 32 - __clz(cost) : 0;
    const int frac = len > 3 ? (int)((cost >> (len - 4)) & 7u) : (int)((cost << (4 - len)) & 7u);
    const int sub = first == 0x7FFFFFFF ? BIN_ORDER_SUB - 1
                                        : (int)(((long long)first * (BIN_ORDER_SUB - 1)) / max(1, nchunks));
    return (BIN_ORDER_FINE - 1 - (len * 8 + frac)) * BIN_ORDER_SUB + sub;
}

__global__ void __launch_bounds__(BIN_ORDER_THREADS) k_bin_order(const __grid_constant__ DrawParams D)
{
    extern __shared__ int cnt[];  // (binsY + 1) x (binsX + 1), then as many cost cells with binCost
    __shared__ uint32_t hist[BIN_ORDER_KEYS];
    __shared__ unsigned long long tot[2];
    const int W = D.binsX + 1, H = D.binsY + 1, nb = D.binsX * D.binsY, tid = threadIdx.x;
    uint32_t *cost = reinterpret_cast<uint32_t *>(cnt + W * H);
    for(int i = tid; i < W * H; i += blockDim.x)
    {
        cnt[i] = D.binDiff[i];
        if(D.binCost) cost[i] = D.binCost[i];
    }
    for(int i = tid; i < BIN_ORDER_KEYS; i += blockDim.x) hist[i] = 0;
    if(tid < 2) tot[tid] = 0ull;
    __syncthreads();
    for(int r = tid; r < H; r += blockDim.x)
    {
        int acc = 0;
        uint32_t cacc = 0u;
        for(int x = 0; x < W; x++)
        {
            cnt[r * W + x] = (acc += cnt[r * W + x]);
            if(D.binCost) cost[r * W + x] = (cacc += cost[r * W + x]);
        }
    }
    __syncthreads();
    for(int c = tid; c < W; c += blockDim.x)
    {
        int acc = 0;
        uint32_t cacc = 0u;
        for(int y = 0; y < H; y++)
        {
            cnt[y * W + c] = (acc += cnt[y * W + c]);
            if(D.binCost) cost[y * W + c] = (cacc += cost[y * W + c]);
        }
    }
    __syncthreads();
    // cost of a bin: its spread triangle area plus its triangle count weighted
    // by the draw's mean area per triangle and bin (equal shares over the
    // draw), or the count alone without the area array
    __shared__ uint32_t nSplit;
    if(tid == 0) nSplit = 0u;
    {
        unsigned long long sc = 0ull, sa = 0ull;
        for(int b = tid; b < nb; b += blockDim.x)
        {
            const int c = (b / D.binsX) * W + b % D.binsX;
            sc += (unsigned long long)max(cnt[c], 0);
            if(D.binCost) sa += cost[c];
        }
        for(int o = 16; o > 0; o >>= 1)
        {
            sc += __shfl_xor_sync(0xFFFFFFFFu, sc, o);
            sa += __shfl_xor_sync(0xFFFFFFFFu, sa, o);
        }
        if((tid & 31) == 0)
        {
            atomicAdd(&tot[0], sc);
            atomicAdd(&tot[1], sa);
        }
        __syncthreads();
    }
    const float perTri = D.binCost && tot[0] ? (float)tot[1] / (float)tot[0] : 0.0f;
    auto value = [&](int b) {
        const int c = (b / D.binsX) * W + b % D.binsX;
        return (float)max(cnt[c], 0) * (D.binCost ? perTri : 1.0f) + (D.binCost ? (float)cost[c] : 0.0f);
    };
    auto key = [&](int b, float v) {
        return bin_order_key(v >= 2147483648.0f ? 0x80000000u : (uint32_t)v, D.binFirst[b], D.nchunks);
    };
    // A bin whose cost exceeds 3/4 of a resident warp's mean share would hold
    // the frame's end on its own: it is queued as two halves (its top and its
    // bottom rows), each ordered by half the cost.  On the 1M-triangle 1080p
    // height field the heaviest bin alone took longer than the warps' mean
    // load (0.73 vs 0.58 ms, instrumented); splitting at 3/4 took k_raster
    // 0.659 -> 0.636 ms (at 1/2: 0.670, 0.65: 0.649, 0.85: 0.648, 1: 0.664).
    const float total = D.binCost ? 2.0f * (float)tot[1] : (float)tot[0];
    const float splitAt = D.binSplit && D.rasterWarps ? 0.75f * total / (float)D.rasterWarps : 3.0e38f;
    for(int b = tid; b < nb; b += blockDim.x)
    {
        const float v = value(b);
        if(v > splitAt)
        {
            atomicAdd(&hist[key(b, 0.5f * v)], 2u);
            atomicAdd(&nSplit, 1u);
        }
        else
            atomicAdd(&hist[key(b, v)], 1u);
    }
    __syncthreads();
    // exclusive scan of the histogram, 'per' consecutive entries per thread
    __shared__ uint32_t warpSum[BIN_ORDER_THREADS / 32];
    {
        const int per = (BIN_ORDER_KEYS + BIN_ORDER_THREADS - 1) / BIN_ORDER_THREADS;
        uint32_t v[8] = {0, 0, 0, 0, 0, 0, 0, 0}, s = 0;
        static_assert((BIN_ORDER_KEYS + BIN_ORDER_THREADS - 1) / BIN_ORDER_THREADS <= 8, "scan entries per thread");
        for(int j = 0; j < per; j++)
        {
            const int i = tid * per + j;
            v[j] = i < BIN_ORDER_KEYS ? hist[i] : 0u;
            s += v[j];
        }
        const int lane = tid & 31, warp = tid >> 5;
        uint32_t incl = s;
        for(int o = 1; o < 32; o <<= 1)
        {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if(lane >= o) incl += u;
        }
        if(lane == 31) warpSum[warp] = incl;
        __syncthreads();
        if(warp == 0)
        {
            uint32_t w = warpSum[lane], wi = w;
            for(int o = 1; o < 32; o <<= 1)
            {
                const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, wi, o);
                if(lane >= o) wi += u;
            }
            warpSum[lane] = wi - w;
        }
        __syncthreads();
        uint32_t run = warpSum[warp] + incl - s;
        for(int j = 0; j < per; j++)
        {
            const int i = tid * per + j;
            if(i < BIN_ORDER_KEYS) hist[i] = run;
            run += v[j];
        }
    }
    __syncthreads();
    for(int b = tid; b < nb; b += blockDim.x)
    {
        const float v = value(b);
        if(v > splitAt)
        {
            const uint32_t pos = atomicAdd(&hist[key(b, 0.5f * v)], 2u);
            D.binOrder[pos] = (uint32_t)b | 1u << 30;
            D.binOrder[pos + 1] = (uint32_t)b | 2u << 30;
        }
        else
        {
            const uint32_t pos = atomicAdd(&hist[key(b, v)], 1u);
            D.binOrder[pos] = (uint32_t)b;
        }
    }
    if(tid == 0) D.binOrder[2 * nb] = (uint32_t)nb + nSplit;
}

// Candidate lists of a single draw's bins: one warp per bin walks the
// super-chunk, chunk and triangle boxes in primitive order -- the walk the
// raster's warp would do -- and writes the triangles whose boxes reach the
// bin.  Without shared memory many more warps are resident than in k_raster,
// which hides the walk's chain of dependent loads; the raster then reads a
// bin's candidates 32 at a time.  A bin with more than binListCap candidates
// stops there with a count above the capacity, and the raster walks it
// itself.  The triangle boxes of up to four hit chunks are loaded together.
// On the 1M-triangle 1080p height field this took ~60 us and made k_raster
// 1.09 -> 1.015 ms.
constexpr int BIN_LIST_WARPS = 8;
__global__ void __launch_bounds__(32 * BIN_LIST_WARPS) k_bin_list(const __grid_constant__ DrawParams D)
{
    const int lane = threadIdx.x & 31;
    const int bin = (int)blockIdx.x * BIN_LIST_WARPS + (int)(threadIdx.x >> 5);
    if(bin >= D.binsX * D.binsY) return;  // whole warps
    const int bx0 = D.binX0 + (bin % D.binsX) * D.binW, by0 = D.binY0 + (bin / D.binsX) * D.binH;
    const int bx1 = bx0 + D.binW, by1 = by0 + D.binH;
    auto hits = [&](int x0, int y0, int x1, int y1) { return x0 < x1 && x0 < bx1 && x1 > bx0 && y0 < by1 && y1 > by0; };
    uint32_t *out = D.binList + (size_t)bin * D.binListCap;
    uint32_t n = 0;
    for(int sb = 0; sb < D.nsuper; sb += 32)
    {
        int4 s = make_int4(0, 0, 0, 0);
        if(sb + lane < D.nsuper) s = D.superBox[sb + lane];
        unsigned superHits = __ballot_sync(0xFFFFFFFFu, sb + lane < D.nsuper && hits(s.x, s.y, s.z, s.w));
        while(superHits)
        {
            const int sc = sb + __ffs(superHits) - 1;
            superHits &= superHits - 1;
            for(int cw = 0; cw < SUPER; cw += 32)
            {
                const int c = sc * SUPER + cw + lane;
                short4 cb = make_short4(0, 0, 0, 0);
                if(c < D.nchunks) cb = D.chunkBox[c];
                unsigned chunkHits = __ballot_sync(0xFFFFFFFFu, c < D.nchunks && hits(cb.x, cb.y, cb.z, cb.w));
                while(chunkHits)
                {
                    int ch[4];
                    short4 tb[4];
#pragma unroll
                    for(int j = 0; j < 4; j++)
                    {
                        ch[j] = -1;
                        if(chunkHits)
                        {
                            ch[j] = sc * SUPER + cw + __ffs(chunkHits) - 1;
                            chunkHits &= chunkHits - 1;
                        }
                        tb[j] = make_short4(0, 0, 0, 0);
                        const uint32_t tri = (uint32_t)ch[j] * CHUNK + lane;
                        if(ch[j] >= 0 && tri < D.count) tb[j] = D.triBox[tri];
                    }
#pragma unroll
                    for(int j = 0; j < 4; j++)
                    {
                        if(ch[j] < 0) break;  // warp-uniform
                        const uint32_t tri = (uint32_t)ch[j] * CHUNK + lane;
                        const bool th = tri < D.count && hits(tb[j].x, tb[j].y, tb[j].z, tb[j].w);
                        const unsigned b = __ballot_sync(0xFFFFFFFFu, th);
                        const uint32_t pos = n + __popc(b & ((1u << lane) - 1u));
                        if(th && pos < D.binListCap) out[pos] = tri;
                        n += __popc(b);
                        if(n > D.binListCap) goto counted;  // the raster walks this bin itself
                    }
                }
            }
        }
    }
counted:
    if(lane == 0) D.binListCount[bin] = n;
}

#endif  // SWGB_RASTER_TU

// ------------------------------------------------------------------------
// SamplerCore 16-bit path for R8G8B8A8_UNORM (src/Pipeline/SamplerCore.cpp)
// ------------------------------------------------------------------------

// address() 16-bit (SamplerCore.cpp:2399-2435).  MIRROR_CLAMP_TO_EDGE
// (ADDRESSING_MIRRORONCE: Int4(Abs(u * 2^16)) - 0x8000, saturated to int16,
// + 0x8000) equals CLAMP_TO_EDGE of |u| -- min(trunc(|u| 2^16), 0xFFFF) both
// ways -- except for NaN, which it maps to 0xFFFF (the conversion gives
// 0x80000000, the subtraction wraps it positive): NaN is taken as 1.  Only
// the full-pipeline raster variants (MIRROR_ONCE) carry that mode.
template<bool MIRROR_ONCE>
__device__ __forceinline__ uint32_t address16(float uw, uint32_t mode)
{
    if(mode == SWGB_ADDRESS_CLAMP_TO_EDGE || (MIRROR_ONCE && mode == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE))
    {
        if(MIRROR_ONCE && mode == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE) uw = uw == uw ? fabsf(uw) : 1.0f;
        float c = rmin(rmax(uw, 0.0f), 65535.0f / 65536.0f);
        return (uint32_t)trunc_int(c * 65536.0f) & 0xFFFFu;
    }
    if(mode == SWGB_ADDRESS_MIRRORED_REPEAT)
    {
        int32_t convert = trunc_int(uw * 65536.0f);
        int32_t mirror = (int32_t)((uint32_t)convert << 15) >> 31;
        convert ^= mirror;
        return (uint32_t)convert & 0xFFFFu;
    }
    return (uint32_t)trunc_int(uw * 65536.0f) & 0xFFFFu;
}

// offsetSample (SamplerCore.cpp:278-313)
__device__ __forceinline__ uint32_t offset_sample(uint32_t uvw, uint32_t half, bool wrap, int count)
{
    if(wrap) return (count < 0 ? uvw - half : uvw + half) & 0xFFFFu;
    return count < 0 ? subsat_u16(uvw, half) : addsat_u16(uvw, half);
}

// computeIndices + 8-bit unpack (SamplerCore.cpp:1593-1643,1747-1788): returns the texel as 4 bytes.
// The components of an 8-bit texel as the 16-bit path holds them
// (SamplerCore.cpp:1747-1788): byte << 8 in R, G, B, A order (B8G8R8A8 texels,
// R and B swapped in memory, are put in that order first with texel_order);
// the R, G, B of an sRGB texture become their sRGBtoLinearFF_FF00 entry
// (:1966-1978,2670-2680).
__device__ __forceinline__ uint32_t texel_order(const DrawParams &D)
{
    return D.texBGRA ? 0x3012u : 0x3210u;  // __byte_perm selector
}

__device__ __forceinline__ void texel_components(const DrawParams &D, uint32_t t, uint32_t out[4])
{
#pragma unroll
    for(int c = 0; c < 4; c++) out[c] = ((t >> (8 * c)) & 0xFFu) << 8;
    if(D.texSRGB)
#pragma unroll
        for(int c = 0; c < 3; c++) out[c] = __ldg(D.srgbLut + (out[c] >> 8));
}

// bilinearInterpolate of sRGB texels (SamplerCore.cpp:516-575 after the
// table decode).  Out of line: the raster loop carries it for sRGB textures
// only.
static __device__ __noinline__ void bilinear_srgb(const DrawParams &D, uint32_t t00, uint32_t t10, uint32_t t01, uint32_t t11,
                                                  uint32_t f0u0v, uint32_t f1u0v, uint32_t f0u1v, uint32_t f1u1v, uint32_t out[4])
{
    uint32_t c00[4], c10[4], c01[4], c11[4];
    texel_components(D, t00, c00);
    texel_components(D, t10, c10);
    texel_components(D, t01, c01);
    texel_components(D, t11, c11);
#pragma unroll
    for(int c = 0; c < 4; c++)
    {
        uint32_t a = mulhi_u16(c00[c], f1u1v);
        uint32_t b = mulhi_u16(c10[c], f0u1v);
        uint32_t e = mulhi_u16(c01[c], f1u0v);
        uint32_t g = mulhi_u16(c11[c], f0u0v);
        out[c] = (((a + b) & 0xFFFFu) + ((e + g) & 0xFFFFu)) & 0xFFFFu;
    }
}

__device__ __forceinline__ uint32_t texel_index(const TexLevel &lv, uint32_t u, uint32_t v)
{
    uint32_t xi = mulhi_u16(u, lv.w);
    uint32_t yi = mulhi_u16(v, lv.h);
    return (uint32_t)((int32_t)(int16_t)xi + (int32_t)(int16_t)yi * (int32_t)(int16_t)lv.pitch);  // pmaddwd
}

__device__ __forceinline__ uint32_t texel_rgba8(const TexLevel &lv, uint32_t u, uint32_t v)
{
    return __ldg((const uint32_t *)lv.buf + texel_index(lv, u, v));
}

// MulHigh of component c of an 8-bit texel as the 16-bit path holds it
// (byte << 8) and a 16-bit weight f: (byte << 8) * f >> 16 = byte * f >> 8,
// the high word of (byte << 24) * f.
__device__ __forceinline__ uint32_t texel_mulhi(uint32_t t, int c, uint32_t f)
{
    return __umulhi(__byte_perm(t, 0u, 0x0444u | (uint32_t)c << 12), f);
}

// bilinearInterpolate of four unsigned 8-bit texels (SamplerCore.cpp:516-575):
// weights from the low 16 bits of u0 * width and v0 * height; the four
// products summed modulo 2^16 (the reference adds them in pairs, each sum
// wrapped to 16 bits).
__device__ __forceinline__ void bilinear8(const TexLevel &lv, uint32_t u0, uint32_t v0, uint32_t t00, uint32_t t10, uint32_t t01,
                                          uint32_t t11, uint32_t out[4])
{
    uint32_t f0u = (u0 * lv.w) & 0xFFFFu, f0v = (v0 * lv.h) & 0xFFFFu;
    uint32_t f1u = (~f0u) & 0xFFFFu, f1v = (~f0v) & 0xFFFFu;
    uint32_t f0u0v = mulhi_u16(f0u, f0v), f1u0v = mulhi_u16(f1u, f0v);
    uint32_t f0u1v = mulhi_u16(f0u, f1v), f1u1v = mulhi_u16(f1u, f1v);
#pragma unroll
    for(int c = 0; c < 4; c++)
        out[c] = (texel_mulhi(t00, c, f1u1v) + texel_mulhi(t10, c, f0u1v) + texel_mulhi(t01, c, f1u0v) + texel_mulhi(t11, c, f0u0v)) &
                 0xFFFFu;
}

// Both levels of a trilinear sample of a linear-filtered 8-bit texture
// without sRGB decoding (sampleQuad2D at int(lod) and int(lod) + 1,
// SamplerCore.cpp:324-379,668-909): the eight texel addresses first, then
// the eight loads together, so the sample waits for memory once.
template<bool MIRROR_ONCE>
__device__ __forceinline__ void sample_trilinear8(const DrawParams &D, float u, float v, float lod, uint32_t c[4], uint32_t cc[4],
                                                  uint32_t &lvMask)
{
    const int ilod = trunc_int(lod);  // selectMipmap, MIPMAP_LINEAR (:2357-2379)
    const int top = D.levelCount - 1;
    const int la = ilod < 0 ? 0 : (ilod > top ? top : ilod);
    const int lb = ilod + 1 < 0 ? 0 : (ilod + 1 > top ? top : ilod + 1);
    lvMask |= (1u << la) | (1u << lb);
    const TexLevel &A = D.lv[la], &B = D.lv[lb];
    const uint32_t uu = address16<MIRROR_ONCE>(u, D.addrU);
    const uint32_t vv = address16<MIRROR_ONCE>(v, D.addrV);
    const bool wu = D.addrU == SWGB_ADDRESS_REPEAT, wv = D.addrV == SWGB_ADDRESS_REPEAT;
    const uint32_t au0 = offset_sample(uu, A.uHalf, wu, -1), av0 = offset_sample(vv, A.vHalf, wv, -1);
    const uint32_t au1 = offset_sample(uu, A.uHalf, wu, +1), av1 = offset_sample(vv, A.vHalf, wv, +1);
    const uint32_t bu0 = offset_sample(uu, B.uHalf, wu, -1), bv0 = offset_sample(vv, B.vHalf, wv, -1);
    const uint32_t bu1 = offset_sample(uu, B.uHalf, wu, +1), bv1 = offset_sample(vv, B.vHalf, wv, +1);
    const uint32_t *pa = (const uint32_t *)A.buf, *pb = (const uint32_t *)B.buf;
    const uint32_t ia00 = texel_index(A, au0, av0), ia10 = texel_index(A, au1, av0);
    const uint32_t ia01 = texel_index(A, au0, av1), ia11 = texel_index(A, au1, av1);
    const uint32_t ib00 = texel_index(B, bu0, bv0), ib10 = texel_index(B, bu1, bv0);
    const uint32_t ib01 = texel_index(B, bu0, bv1), ib11 = texel_index(B, bu1, bv1);
    const uint32_t ta00 = __ldg(pa + ia00), ta10 = __ldg(pa + ia10), ta01 = __ldg(pa + ia01), ta11 = __ldg(pa + ia11);
    const uint32_t tb00 = __ldg(pb + ib00), tb10 = __ldg(pb + ib10), tb01 = __ldg(pb + ib01), tb11 = __ldg(pb + ib11);
    bilinear8(A, au0, av0, ta00, ta10, ta01, ta11, c);
    bilinear8(B, bu0, bv0, tb00, tb10, tb01, tb11, cc);
    if(D.texBGRA)
    {
        // B8G8R8A8 texels: the filter works per component, so R and B swap
        // after it rather than in each texel
        uint32_t s = c[0]; c[0] = c[2]; c[2] = s;
        s = cc[0]; cc[0] = cc[2]; cc[2] = s;
    }
}

// sample_trilinear8 plus the trilinear blend and the 1/0xFF00 scale for the
// common state -- R8G8B8A8_UNORM, REPEAT on u and v, every level below 2^15
// texels wide, high and pitched -- with the address modes and the texel order
// fixed: address16 of REPEAT and the wrapping offsetSample inline (the same
// arithmetic), and the level choice and texel index without the out-of-range
// paths that state excludes.  Compiled into the raster variants without depth
// rejection only (TEXFAST): on the 1M-triangle height field it took k_raster
// from 0.951 to 0.898 ms, while in the rejection variants the second sampler
// copy cost the atlas 3%.
__device__ __forceinline__ void sample_trilinear8_repeat(const DrawParams &D, float u, float v, float lod, float out[4],
                                                         uint32_t &lvMask)
{
    // lod comes from implicit_lod: its selects return minLod or maxLod for a
    // NaN or out-of-range value, and the host clamps both into [0, 13] (a NaN
    // bound truncates to level 0), so ilod is never negative
    const int ilod = __float2int_rz(lod);
    const int top = D.levelCount - 1;
    const int la = ilod > top ? top : ilod;
    const int lb = ilod + 1 > top ? top : ilod + 1;
    lvMask |= (1u << la) | (1u << lb);
    const TexLevel &A = D.lv[la], &B = D.lv[lb];
    const uint32_t uu = (uint32_t)trunc_int(u * 65536.0f) & 0xFFFFu;
    const uint32_t vv = (uint32_t)trunc_int(v * 65536.0f) & 0xFFFFu;
    const uint32_t au0 = (uu - A.uHalf) & 0xFFFFu, av0 = (vv - A.vHalf) & 0xFFFFu;
    const uint32_t au1 = (uu + A.uHalf) & 0xFFFFu, av1 = (vv + A.vHalf) & 0xFFFFu;
    const uint32_t bu0 = (uu - B.uHalf) & 0xFFFFu, bv0 = (vv - B.vHalf) & 0xFFFFu;
    const uint32_t bu1 = (uu + B.uHalf) & 0xFFFFu, bv1 = (vv + B.vHalf) & 0xFFFFu;
    // texel_index with width, height and pitch below 2^15 (the state's
    // condition): MulHigh by the width / height, and the 16-bit row product,
    // never leave the int16 range
    const uint32_t axa0 = au0 * A.w >> 16, axa1 = au1 * A.w >> 16, aya0 = (av0 * A.h >> 16) * A.pitch, aya1 = (av1 * A.h >> 16) * A.pitch;
    const uint32_t bxa0 = bu0 * B.w >> 16, bxa1 = bu1 * B.w >> 16, bya0 = (bv0 * B.h >> 16) * B.pitch, bya1 = (bv1 * B.h >> 16) * B.pitch;
    const uint32_t *pa = (const uint32_t *)A.buf, *pb = (const uint32_t *)B.buf;
    const uint32_t ta00 = __ldg(pa + axa0 + aya0), ta10 = __ldg(pa + axa1 + aya0);
    const uint32_t ta01 = __ldg(pa + axa0 + aya1), ta11 = __ldg(pa + axa1 + aya1);
    const uint32_t tb00 = __ldg(pb + bxa0 + bya0), tb10 = __ldg(pb + bxa1 + bya0);
    const uint32_t tb01 = __ldg(pb + bxa0 + bya1), tb11 = __ldg(pb + bxa1 + bya1);
    uint32_t c[4], cc[4];
    bilinear8(A, au0, av0, ta00, ta10, ta01, ta11, c);
    bilinear8(B, bu0, bv0, tb00, tb10, tb01, tb11, cc);
    const uint32_t utri = (uint32_t)__float2int_rz(lod * 65536.0f) & 0xFFFFu;  // sampleFilter trilinear blend (:324-379)
    const float scale = 1.0f / 65280.0f;
#pragma unroll
    for(int j = 0; j < 4; j++)
        out[j] = __uint2float_rn(((c[j] * (utri ^ 0xFFFFu) >> 16) + (cc[j] * utri >> 16)) & 0xFFFFu) * scale;
}

// sampleQuad2D for one lane, 16-bit channel values c << 8 (SamplerCore.cpp:668-909).
template<bool MIRROR_ONCE>
__device__ __forceinline__ void sample_quad_2d(const DrawParams &D, float u, float v, float lod, int second, uint32_t out[4], uint32_t &lvMask)
{
    int ilod = D.mipLinear ? trunc_int(lod) : round_int(lod);  // selectMipmap (:2357-2379)
    int li = ilod + second;
    li = li < 0 ? 0 : (li > D.levelCount - 1 ? D.levelCount - 1 : li);
    lvMask |= 1u << li;
    const TexLevel &lv = D.lv[li];
    uint32_t uu = address16<MIRROR_ONCE>(u, D.addrU);
    uint32_t vv = address16<MIRROR_ONCE>(v, D.addrV);
    if(!D.texLinear)
    {
        texel_components(D, __byte_perm(texel_rgba8(lv, uu, vv), 0u, texel_order(D)), out);
        return;
    }
    bool wu = D.addrU == SWGB_ADDRESS_REPEAT, wv = D.addrV == SWGB_ADDRESS_REPEAT;
    uint32_t u0 = offset_sample(uu, lv.uHalf, wu, -1), v0 = offset_sample(vv, lv.vHalf, wv, -1);
    uint32_t u1 = offset_sample(uu, lv.uHalf, wu, +1), v1 = offset_sample(vv, lv.vHalf, wv, +1);
    uint32_t t00 = texel_rgba8(lv, u0, v0), t10 = texel_rgba8(lv, u1, v0);
    uint32_t t01 = texel_rgba8(lv, u0, v1), t11 = texel_rgba8(lv, u1, v1);
    {
        const uint32_t sel = texel_order(D);
        t00 = __byte_perm(t00, 0u, sel);
        t10 = __byte_perm(t10, 0u, sel);
        t01 = __byte_perm(t01, 0u, sel);
        t11 = __byte_perm(t11, 0u, sel);
    }
    if(D.texSRGB)
    {
        uint32_t f0u = (u0 * lv.w) & 0xFFFFu, f0v = (v0 * lv.h) & 0xFFFFu;
        uint32_t f1u = (~f0u) & 0xFFFFu, f1v = (~f0v) & 0xFFFFu;
        uint32_t o[4];  // a temporary: the caller's array stays in registers
        bilinear_srgb(D, t00, t10, t01, t11, mulhi_u16(f0u, f0v), mulhi_u16(f1u, f0v), mulhi_u16(f0u, f1v), mulhi_u16(f1u, f1v), o);
#pragma unroll
        for(int k = 0; k < 4; k++) out[k] = o[k];
        return;
    }
    bilinear8(lv, u0, v0, t00, t10, t01, t11, out);  // bilinearInterpolate, unsigned 8-bit components (:516-575)
}

// Implicit LOD of computeLod2D (SamplerCore.cpp:1376-1422) from lanes 0, 1, 2
// of the quad, plus mipLodBias and the [minLod, maxLod] clamp (:116-157).
__device__ __forceinline__ float implicit_lod(const DrawParams &D, const float u[4], const float v[4])
{
    if(D.minLod == D.maxLod) return D.minLod;
    float dudx = u[1] - u[0], dudy = u[2] - u[0];
    float dvdx = v[1] - v[0], dvdy = v[2] - v[0];
    float a = dudx * D.texW, b = dudy * D.texW, c = dvdx * D.texH, e = dvdy * D.texH;
    a = a * a; b = b * b; c = c * c; e = e * e;
    float lod = log2sqrt(rmax(a + c, b + e));
    lod = lod + D.lodBias;
    lod = rmax(lod, D.minLod);
    return rmin(lod, D.maxLod);
}

// sampleTexture128 on the 16-bit path (SamplerCore.cpp:59-253) for lane 'lane'
// of a quad; the result is scaled by 1 / 0xFF00 (getComponentScale).
template<bool MIRROR_ONCE, bool TEXFAST = false>
__device__ __forceinline__ void sample_texture_lane(const DrawParams &D, float lod, float ul, float vl, float out[4],
                                                    uint32_t &lvMask)
{
    if(TEXFAST && !MIRROR_ONCE && D.texRepeatTrilinear)
    {
        sample_trilinear8_repeat(D, ul, vl, lod, out, lvMask);
        return;
    }
    uint32_t c[4], cc[4] = {0u, 0u, 0u, 0u};
    if(D.mipLinear && D.texLinear && !D.texSRGB)
        sample_trilinear8<MIRROR_ONCE>(D, ul, vl, lod, c, cc, lvMask);
    else
    {
        const int levels = D.mipLinear ? 2 : 1;
#pragma unroll 1
        for(int second = 0; second < levels; second++)
        {
            uint32_t t[4];
            sample_quad_2d<MIRROR_ONCE>(D, ul, vl, lod, second, t, lvMask);
#pragma unroll
            for(int k = 0; k < 4; k++)
            {
                if(second) cc[k] = t[k]; else c[k] = t[k];
            }
        }
    }
    if(D.mipLinear)  // sampleFilter trilinear blend (:324-379)
    {
        const uint32_t utri = (uint32_t)trunc_int(lod * 65536.0f) & 0xFFFFu;
#pragma unroll
        for(int k = 0; k < 4; k++) c[k] = (mulhi_u16(c[k], (~utri) & 0xFFFFu) + mulhi_u16(cc[k], utri)) & 0xFFFFu;
    }
    const float scale = 1.0f / 65280.0f;
#pragma unroll
    for(int k = 0; k < 4; k++) out[k] = __uint2float_rn(c[k]) * scale;
}

// ---- fp32 filtering path for R16G16B16A16_SFLOAT / R32G32B32A32_SFLOAT ----------

// address() for normalized float coordinates (SamplerCore.cpp:2463-2638).
__device__ __forceinline__ void address_float(const DrawParams &D, float coord, uint32_t mode, int dim, int32_t &x0, int32_t &x1, float &f)
{
    const float one = __int_as_float(0x3F7FFFFF);
    if(mode == SWGB_ADDRESS_CLAMP_TO_EDGE)
        coord = rmin(rmax(coord, 0.0f), one);
    else if(mode == SWGB_ADDRESS_MIRRORED_REPEAT)
    {
        coord = coord * 0.5f;
        coord = 2.0f * fabsf(coord - rintf(coord));
        coord = rmin(coord, one);
    }
    else if(mode == SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE)
        coord = rmin(fabsf(coord), one);
    else if(mode != SWGB_ADDRESS_CLAMP_TO_BORDER)  // a border axis keeps the coordinate
        coord = rmin(coord - floorf(coord), one);  // Float4 Frac (LLVMReactor.cpp:3252-3275)
    coord = coord * (float)dim;
    if(mode == SWGB_ADDRESS_CLAMP_TO_BORDER)
    {
        // out-of-range texel coordinates become -1 and read the border
        if(!D.texLinear)
            x0 = trunc_int(floorf(coord));
        else
        {
            coord = coord - 0.5f;
            const float fl = floorf(coord);
            x0 = trunc_int(fl);
            f = coord - fl;
        }
        x1 = x0 + 1;
        if(x0 < 0 || x0 >= dim) x0 = -1;
        if(x1 < 0 || x1 >= dim) x1 = -1;
        if(!D.texLinear) f = 0.0f;
        return;
    }
    if(!D.texLinear)
    {
        x0 = trunc_int(coord);
        x1 = x0 + 1;
        f = 0.0f;
        return;
    }
    coord = coord - 0.5f;
    const float fl = floorf(coord);
    x0 = trunc_int(fl);
    f = coord - fl;
    x1 = x0 + 1;
    if(mode == SWGB_ADDRESS_REPEAT)
    {
        if(x0 < 0) x0 = dim - 1;
        if(!(x1 < dim)) x1 = 0;
    }
    else
    {
        x0 = max(x0, 0);
        x1 = min(x1, dim - 1);
    }
}

__device__ __forceinline__ float4 texel_float(const DrawParams &D, const TexLevel &lv, int32_t index)
{
    if(D.texFloat == 0)
    {
        // an 8-bit texture on the fp32 path (border addressing): the 16-bit
        // path's components as floats (SamplerCore.cpp:2215-2245)
        uint32_t c[4];
        texel_components(D, __byte_perm(__ldg((const uint32_t *)lv.buf + (uint32_t)index), 0u, texel_order(D)), c);
        return make_float4((float)c[0], (float)c[1], (float)c[2], (float)c[3]);
    }
    if(D.texFloat == 2) return __ldg((const float4 *)lv.buf + (uint32_t)index);
    const uint2 h = __ldg((const uint2 *)lv.buf + (uint32_t)index);
    return make_float4(half_bits_to_float(h.x & 0xFFFFu), half_bits_to_float(h.x >> 16),
                       half_bits_to_float(h.y & 0xFFFFu), half_bits_to_float(h.y >> 16));
}

// sampleFloat2D for one lane (SamplerCore.cpp:1155-1248).  BORDER: the
// full-pipeline raster variants, which carry CLAMP_TO_BORDER addressing.
template<bool BORDER>
__device__ __forceinline__ float4 sample_float_2d(const DrawParams &D, float u, float v, float lod, int second, uint32_t &lvMask)
{
    int ilod = D.mipLinear ? trunc_int(lod) : round_int(lod);
    int li = ilod + second;
    li = li < 0 ? 0 : (li > D.levelCount - 1 ? D.levelCount - 1 : li);
    lvMask |= 1u << li;
    const TexLevel &lv = D.lv[li];
    int32_t x0, x1, y0, y1;
    float fu, fv;
    address_float(D, u, D.addrU, (int)lv.w, x0, x1, fu);
    address_float(D, v, D.addrV, (int)lv.h, y0, y1, fv);
    const int32_t pitch = (int32_t)lv.pitch;
    if(BORDER && D.border)
    {
        // sampleTexel with border addressing (SamplerCore.cpp:2093-2110,
        // 1645-1677, 2290-2355): a texel with a -1 coordinate reads index 0
        // and is replaced by the border colour
        const float4 bc = make_float4(D.borderColor[0], D.borderColor[1], D.borderColor[2], D.borderColor[3]);
        auto fetch = [&](int32_t x, int32_t y) {
            const bool valid = x >= 0 && y >= 0;
            const float4 t = texel_float(D, lv, valid ? x + y * pitch : 0);
            return valid ? t : bc;
        };
        if(!D.texLinear) return fetch(x0, y0);
        const float4 c00 = fetch(x0, y0), c10 = fetch(x1, y0), c01 = fetch(x0, y1), c11 = fetch(x1, y1);
        float4 a, b, o;
        a.x = c00.x + fu * (c10.x - c00.x); a.y = c00.y + fu * (c10.y - c00.y);
        a.z = c00.z + fu * (c10.z - c00.z); a.w = c00.w + fu * (c10.w - c00.w);
        b.x = c01.x + fu * (c11.x - c01.x); b.y = c01.y + fu * (c11.y - c01.y);
        b.z = c01.z + fu * (c11.z - c01.z); b.w = c01.w + fu * (c11.w - c01.w);
        o.x = a.x + fv * (b.x - a.x); o.y = a.y + fv * (b.y - a.y);
        o.z = a.z + fv * (b.z - a.z); o.w = a.w + fv * (b.w - a.w);
        return o;
    }
    y0 *= pitch;
    if(!D.texLinear) return texel_float(D, lv, x0 + y0);
    y1 *= pitch;
    const float4 c00 = texel_float(D, lv, x0 + y0), c10 = texel_float(D, lv, x1 + y0);
    const float4 c01 = texel_float(D, lv, x0 + y1), c11 = texel_float(D, lv, x1 + y1);
    float4 a, b, o;
    a.x = c00.x + fu * (c10.x - c00.x); a.y = c00.y + fu * (c10.y - c00.y);
    a.z = c00.z + fu * (c10.z - c00.z); a.w = c00.w + fu * (c10.w - c00.w);
    b.x = c01.x + fu * (c11.x - c01.x); b.y = c01.y + fu * (c11.y - c01.y);
    b.z = c01.z + fu * (c11.z - c01.z); b.w = c01.w + fu * (c11.w - c01.w);
    o.x = a.x + fv * (b.x - a.x); o.y = a.y + fv * (b.y - a.y);
    o.z = a.z + fv * (b.z - a.z); o.w = a.w + fv * (b.w - a.w);
    return o;
}

// sampleFloatFilter (SamplerCore.cpp:1061-1083): trilinear blend by the scalar
// Frac of the LOD (x86 SSE4.1: lod - floor(lod)).
// Out of line: the raster kernels carry both filtering paths, and the fp32 one
// inlined would crowd the UNORM8 path's code in the loop.
template<bool BORDER>
static __device__ __noinline__ void sample_float_lane(const DrawParams &D, float lod, float ul, float vl, float out[4], uint32_t &lvMask)
{
    float4 c = sample_float_2d<BORDER>(D, ul, vl, lod, 0, lvMask);
    if(D.mipLinear)
    {
        const float4 cc = sample_float_2d<BORDER>(D, ul, vl, lod, 1, lvMask);
        const float fr = lod - floorf(lod);
        c.x = (cc.x - c.x) * fr + c.x;
        c.y = (cc.y - c.y) * fr + c.y;
        c.z = (cc.z - c.z) * fr + c.z;
        c.w = (cc.w - c.w) * fr + c.w;
    }
    if(BORDER && D.texFloat == 0)  // normalized 8-bit texels: 1 / getComponentScale() (SamplerCore.cpp:200-209)
    {
        const float s = 1.0f / 65280.0f;
        c.x = c.x * s; c.y = c.y * s; c.z = c.z * s; c.w = c.w * s;
    }
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
}

// ------------------------------------------------------------------------
// Raster stage
// ------------------------------------------------------------------------

__device__ __forceinline__ float blend_factor(uint32_t f, const float *src, const float *dst, int comp)
{
    bool alpha = comp == 3;
    switch(f)
    {
    case SWGB_BLEND_ZERO: return 0.0f;
    case SWGB_BLEND_ONE: return 1.0f;
    case SWGB_BLEND_SRC_COLOR: return alpha ? src[3] : src[comp];
    case SWGB_BLEND_ONE_MINUS_SRC_COLOR: return 1.0f - (alpha ? src[3] : src[comp]);
    case SWGB_BLEND_DST_COLOR: return alpha ? dst[3] : dst[comp];
    case SWGB_BLEND_ONE_MINUS_DST_COLOR: return 1.0f - (alpha ? dst[3] : dst[comp]);
    case SWGB_BLEND_SRC_ALPHA: return src[3];
    case SWGB_BLEND_ONE_MINUS_SRC_ALPHA: return 1.0f - src[3];
    case SWGB_BLEND_DST_ALPHA: return dst[3];
    case SWGB_BLEND_ONE_MINUS_DST_ALPHA: return 1.0f - dst[3];
    default: return 0.0f;
    }
}

__device__ __forceinline__ float blend_op(uint32_t op, float s, float sf, float d, float df)
{
    switch(op)
    {
    case SWGB_BLEND_OP_ADD: return s * sf + d * df;
    case SWGB_BLEND_OP_SUBTRACT: return s * sf - d * df;
    case SWGB_BLEND_OP_REVERSE_SUBTRACT: return d * df - s * sf;
    case SWGB_BLEND_OP_MIN: return rmin(s, d);
    case SWGB_BLEND_OP_MAX: return rmax(s, d);
    case OP_SRC_EXT: return s;
    case OP_DST_EXT: return d;
    case OP_ZERO_EXT: return 0.0f;
    default: return s;
    }
}

// alphaBlend with any factors and ops (PixelRoutine.cpp:1653-1961).  Out of
// line, like every rarely taken path of the raster loop.
static __device__ __noinline__ void blend_generic(const DrawParams &D, const float col[4], const float dst[4], float out[4])
{
    float sf[4], df[4];
#pragma unroll
    for(int c = 0; c < 3; c++)
    {
        sf[c] = blend_factor(D.srcC, col, dst, c);
        df[c] = blend_factor(D.dstC, col, dst, c);
    }
    sf[3] = blend_factor(D.srcA, col, dst, 3);
    df[3] = blend_factor(D.dstA, col, dst, 3);
#pragma unroll
    for(int c = 0; c < 3; c++) out[c] = blend_op(D.opC, col[c], sf[c], dst[c], df[c]);
    out[3] = blend_op(D.opA, col[3], sf[3], dst[3], df[3]);
}

// sRGB colour attachments: decode of the blend's destination read, encode
// before the write (ShaderCore.cpp:914-930).  Out of line: full-pipeline
// kernels only.
static __device__ __noinline__ void srgb_decode3(float v[4])
{
#pragma unroll
    for(int c = 0; c < 3; c++) v[c] = srgb_to_linear(v[c]);
}
static __device__ __noinline__ void srgb_encode3(float v[4])
{
#pragma unroll
    for(int c = 0; c < 3; c++) v[c] = linear_to_srgb(v[c]);
}

// The depth a fragment tests and writes: z itself for D32_SFLOAT; for
// D16_UNORM Min(Max(Round(z * 0xFFFF), 0), 0xFFFF), compared against the
// stored 16-bit value as a float and written back as that integer
// (PixelRoutine.cpp:506-510,687-713).  Monotonic in z.
template<bool FULL>
__device__ __forceinline__ float depth_value(const DrawParams &D, float z)
{
    if(!FULL || !D.depth16) return z;
    return fminf(fmaxf(rintf(z * 65535.0f), 0.0f), 65535.0f);
}

// Depth bounds test of the stored depth (depthBoundsTest16/32F,
// PixelRoutine.cpp:576-640): minDepthBounds <= z <= maxDepthBounds, D16_UNORM
// values scaled by 1 / 0xFFFF; applied after the depth test, on the value the
// sample found.
__device__ __forceinline__ bool bounds_pass(const DrawParams &D, float stored)
{
    const float z = D.depth16 ? stored * (1.0f / 0xFFFF) : stored;
    return D.minBounds <= z && z <= D.maxBounds;
}

// Stencil test of face f (PixelRoutine.cpp:360-449): (reference & compareMask)
// op (stored & compareMask), unsigned.
__device__ __forceinline__ bool stencil_pass(const DrawParams &D, int f, uint32_t stored)
{
    const uint32_t m = D.sCompareMask[f] & 0xFFu;
    const uint32_t r = D.sReference[f] & m, v = stored & m;
    switch(D.sCompareOp[f])
    {
    case SWGB_COMPARE_NEVER: return false;
    case SWGB_COMPARE_LESS: return r < v;
    case SWGB_COMPARE_EQUAL: return r == v;
    case SWGB_COMPARE_LESS_OR_EQUAL: return r <= v;
    case SWGB_COMPARE_GREATER: return r > v;
    case SWGB_COMPARE_NOT_EQUAL: return r != v;
    case SWGB_COMPARE_GREATER_OR_EQUAL: return r >= v;
    default: return true;
    }
}

// A stencil operation on a stored byte (PixelRoutine.cpp:862-895).
__device__ __forceinline__ uint32_t stencil_op(const DrawParams &D, int f, uint32_t op, uint32_t v)
{
    switch(op)
    {
    case SWGB_STENCIL_OP_ZERO: return 0u;
    case SWGB_STENCIL_OP_REPLACE: return D.sReference[f] & 0xFFu;
    case SWGB_STENCIL_OP_INCREMENT_AND_CLAMP: return v < 255u ? v + 1u : 255u;
    case SWGB_STENCIL_OP_DECREMENT_AND_CLAMP: return v > 0u ? v - 1u : 0u;
    case SWGB_STENCIL_OP_INVERT: return (~v) & 0xFFu;
    case SWGB_STENCIL_OP_INCREMENT_AND_WRAP: return (v + 1u) & 0xFFu;
    case SWGB_STENCIL_OP_DECREMENT_AND_WRAP: return (v - 1u) & 0xFFu;
    default: return v;  // KEEP
    }
}

// Stencil test, then the write-back of the sample's new stored value: failOp
// where the stencil test failed, depthFailOp where the depth (and bounds) test
// failed, passOp else, through the write mask (writeStencil :754-860).  Out of
// line: only draws with a stencil attachment take it.
static __device__ __noinline__ bool stencil_resolve(const DrawParams &D, uint8_t *sv, int f, bool depthPass)
{
    const uint32_t v = *sv;
    const bool sp = stencil_pass(D, f, v);
    if(D.stencilWrite)
    {
        const uint32_t op = !sp ? D.sFailOp[f] : (!depthPass ? D.sDepthFailOp[f] : D.sPassOp[f]);
        const uint32_t wm = D.sWriteMask[f] & 0xFFu;
        *sv = (uint8_t)((stencil_op(D, f, op, v) & wm) | (v & ~wm));
    }
    return sp;
}

__device__ __forceinline__ bool depth_pass(uint32_t op, float zb, float z)
{
    switch(op)
    {
    case SWGB_COMPARE_NEVER: return false;
    case SWGB_COMPARE_LESS: return !(zb <= z);
    case SWGB_COMPARE_EQUAL: return zb == z;
    case SWGB_COMPARE_LESS_OR_EQUAL: return !(zb < z);
    case SWGB_COMPARE_GREATER: return zb < z;
    case SWGB_COMPARE_NOT_EQUAL: return !(zb == z);
    case SWGB_COMPARE_GREATER_OR_EQUAL: return zb <= z;
    default: return true;
    }
}

// ------------------------------------------------------------------------
// Raster stage
// ------------------------------------------------------------------------

// Per-triangle plane-equation floats staged for a batch:
// x0, y0, z(A,B,C), w(A,B,C), V[k](A,B,C).


// 32-bit words per pixel of a colour attachment: R8G8B8A8_UNORM,
// R16G16B16A16_SFLOAT, R32G32B32A32_SFLOAT.
// R8G8B8A8_UNORM, R16G16B16A16_SFLOAT, R32G32B32A32_SFLOAT, B8G8R8A8_UNORM.
enum { CF_RGBA8 = 0, CF_RGBA16F = 1, CF_RGBA32F = 2, CF_BGRA8 = 3, NCF = 4 };
__host__ __device__ constexpr bool cf_unorm8(int cf) { return cf == CF_RGBA8 || cf == CF_BGRA8; }
__host__ __device__ constexpr int color_words(int cf) { return cf_unorm8(cf) ? 1 : (cf == CF_RGBA16F ? 2 : 4); }

// Shared memory of one warp: its bin's depth and colour, the staged batch,
// and its ordered candidate list.
// BW x BH is the bin's shape in pixels (powers of two, BH even).  FULL: the
// kernel carries the whole per-sample pipeline -- D16_UNORM depth (the staged
// depth then holds its integers), depth bias, the depth bounds test and the
// stencil test; without it those paths are compiled out.
// Shared-memory copies by the asynchronous copy unit (cp.async): the copy is
// issued and the thread goes on; cp_async_wait_all waits for its own copies.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// A batch's live pixels are queued (at most 31 left over plus the 4 pixels of
// each of a quad round's 32 quads) and shaded 32 at a time.
constexpr int PIXQ = 31 + 4 * 32 + 1;

template<int CF, int MS, int BW = BIN, int BH = BIN, bool FULL = false>
struct __align__(16) RasterShared {  // 16: the warps' copies sit back to back and take float4 / uint4 accesses
    float depth[MS][BW * BH];
    uint32_t color[MS][BW * BH * color_words(CF)];
    float4 planeA[BATCH][PLANES_STORED / 4];  // the triangle's plane record, copied from the setup stage
    // per-triangle rows padded to odd word strides: lanes reading different
    // triangles' rows fall in different banks
    uint32_t span[BATCH][MS][BH + 1];  // left | right << 16 per sample and bin row
    int16_t qx0[BATCH][BH / 2 + 2];    // first quad x per quad row of the triangle
    uint16_t qpre[BATCH][BH / 2 + 3];  // prefix of quads per quad row
    int8_t qr0[BATCH];                 // first quad row of the triangle in the bin
    int8_t nqr[BATCH];                 // quad rows of the triangle in the bin
    int triList[2 * BATCH];
    uint32_t pixq[PIXQ];               // live pixels waiting for shading, in primitive order (pix_entry)
    int8_t front[BATCH];               // the triangle faces front (stencil state [0]) or back ([1])
    uint8_t owner[32];                 // quad round: the batch lane whose slots start at window position p
    uint8_t stencil[FULL ? MS : 1][FULL ? BW * BH : 4];  // the bin's stencil values (stencil test active)
    static constexpr int kSamples = MS;
    static constexpr int kBW = BW, kBH = BH;
    static constexpr bool kFull = FULL;
};


// The span rows of triangle t inside bin rows [rowLo, rowHi) by the reference's
// edge DDA, for triangles whose rows did not fit the setup stage's span
// scratch (SetupRoutine::edge, src/Pipeline/SetupRoutine.cpp:550-621).  Out of
// line: it is rare, and inlined it would crowd the raster loop's code.
template<class SH>
__device__ __noinline__ void walk_spans_in_bin(const DrawParams &D, SH &S, int ti, uint32_t t, const TriInfo inf, int by0, int rowLo, int rowHi)
{
    constexpr int MS = SH::kSamples;
    const int n = inf.info & 31, dW = (inf.info >> 5) & 1;
    uint32_t iv0 = 0, iv1 = 0, iv2 = 0;
    int32_t X[MAX_POLY], Y[MAX_POLY];
    if(inf.info & 64)
    {
        for(int i = 0; i < n; i++)
        {
            int2 q = D.poly[(size_t)inf.slot * MAX_POLY + i];
            X[i] = q.x; Y[i] = q.y;
        }
    }
    else
    {
        tri_slots(D, t, iv0, iv1, iv2);
        float4 a = D.ptv[(size_t)iv0 * 4 + 1], b = D.ptv[(size_t)iv1 * 4 + 1], c = D.ptv[(size_t)iv2 * 4 + 1];
        X[0] = __float_as_int(a.x); X[1] = __float_as_int(b.x); X[2] = __float_as_int(c.x);
        Y[0] = __float_as_int(a.y); Y[1] = __float_as_int(b.y); Y[2] = __float_as_int(c.y);
    }
    for(int q = 0; q < MS; q++)
    {
        for(int y = rowLo; y < rowHi; y++) S.span[ti][q][y - by0] = 0u;
        const int32_t dx = MS > 1 ? XF[q] : 0, dy = MS > 1 ? YF[q] : 0;
        for(int i = 0; i < n; i++)
        {
            int ia = i + 1 - dW, ib = i + dW;
            ia = ia == n ? 0 : ia;
            ib = ib == n ? 0 : ib;
            EdgeDDA e;
            if(!edge_setup(D, X[ia] - dx, Y[ia] - dy, X[ib] - dx, Y[ib] - dy, e)) continue;
            int ys = max(e.yMin, rowLo), ye = min(e.yMax, rowHi);
            if(ys >= ye) continue;
            int32_t dd;
            int32_t x = edge_x_at(e, ys, &dd);
            uint16_t *h = reinterpret_cast<uint16_t *>(&S.span[ti][q][0]) + (e.right ? 1 : 0);
            for(int y = ys; y < ye; y++)
            {
                h[2 * (y - by0)] = (uint16_t)clamp_x(D, x);
                x += e.Q;
                dd += e.R;
                int32_t of = (-dd) >> 31;
                dd -= e.D & of;
                x -= of;
            }
        }
    }
}

// R1: one batch triangle -- its span rows inside the bin (from the setup
// stage's span buffer, or the reference DDA when the buffer was full), its
// quad rows, and its plane equations (SetupRoutine.cpp:270-548).  Returns the
// number of quad slots it expands to.
template<class SH>
__device__ int setup_batch_triangle(const DrawParams &D, SH &S, int ti, uint32_t t, int bx0, int by0, int w0 = 0, int w1 = SH::kBH)
{
    // the plane record first: it depends on t only, and arrives while the
    // box, the record and the span rows are fetched
    {
        const float4 *pl = D.planes + (size_t)t * (PLANES_STORED / 4);
        for(int v = 0; v < D.planeVec4; v++) cp_async16(&S.planeA[ti][v], pl + v);
    }
    const short4 box = D.triBox[t];
    const TriInfo inf = D.triInfo[t];
    const int n = inf.info & 31, dW = (inf.info >> 5) & 1;
    S.front[ti] = (int8_t)((inf.info >> 8) & 1);
    constexpr int BW = SH::kBW, BH = SH::kBH;
    // bin rows of the triangle, inside the rows [w0, w1) this warp takes (even)
    const int rowLo = max((int)box.y, by0 + w0), rowHi = min((int)box.w, by0 + w1);
    if(rowLo >= rowHi)
    {
        cp_async_wait_all();  // the plane record's copy lands before the slot is reused
        S.nqr[ti] = 0;
        return 0;
    }
    const int qrA = (rowLo - by0) >> 1, qrB = (rowHi - 1 - by0) >> 1;            // quad rows [qrA, qrB]
    constexpr int MS = SH::kSamples;
    // rows outside [rowLo, rowHi) but inside the quad rows are empty
#pragma unroll
    for(int q = 0; q < MS; q++)
    {
        if(2 * qrA < rowLo - by0) S.span[ti][q][2 * qrA] = 0u;
        if(2 * qrB + 1 >= rowHi - by0) S.span[ti][q][2 * qrB + 1] = 0u;
    }
    if(inf.info & 128)
    {
#pragma unroll
        for(int q = 0; q < MS; q++)
        {
            const uint32_t *sp = D.spans + inf.spanOff + (size_t)q * inf.rows + (rowLo - box.y);
            for(int y = rowLo; y < rowHi; y++) cp_async4(&S.span[ti][q][y - by0], sp + (y - rowLo));
        }
    }
    else
    {
        // span scratch was full at setup: walk the edges here (SetupRoutine::edge)
        walk_spans_in_bin(D, S, ti, t, inf, by0, rowLo, rowHi);
    }
    cp_async_wait_all();
    // quad rows: x range of the row pair over all samples (QuadRasterizer.cpp:96-123), clipped to the bin
    int pre = 0;
    for(int qr = qrA; qr <= qrB; qr++)
    {
        const int k = qr - qrA;
        S.qpre[ti][k] = (uint16_t)pre;
        int xa = 0x7FFF, xb = -1;
#pragma unroll
        for(int q = 0; q < MS; q++)
        {
            uint32_t s0 = S.span[ti][q][2 * qr], s1 = S.span[ti][q][2 * qr + 1];
            int l0 = s0 & 0xFFFF, r0 = s0 >> 16, l1 = s1 & 0xFFFF, r1 = s1 >> 16;
            if(l0 < r0) { xa = min(xa, l0); xb = max(xb, r0); }
            if(l1 < r1) { xa = min(xa, l1); xb = max(xb, r1); }
        }
        int cnt = 0;
        if(xb >= 0)
        {
            xa = max(xa & ~1, bx0);
            xb = min(xb, bx0 + BW);
            cnt = xb > xa ? (xb - xa + 1) >> 1 : 0;
        }
        else
            xa = 0;
        S.qx0[ti][k] = (int16_t)xa;
        pre += cnt;
    }
    S.qpre[ti][qrB - qrA + 1] = (uint16_t)pre;
    S.qr0[ti] = (int8_t)qrA;
    S.nqr[ti] = (int8_t)(qrB - qrA + 1);

    return pre;
}

// Shades one covered pixel (lane i of the 2x2 quad at (qx, y)) of batch
// triangle ti: interpolation (PixelRoutine::quad :124-261), the fixed fragment
// shader with SamplerCore filtering (the LOD comes from lanes 0, 1 and 2 of the
// quad, covered or not, as the reference's 4-wide SIMD computes it), and the
// UNORM clamp (PixelProgram::clampColor).
template<int CF, bool TEXFAST, class SH>
__device__ __forceinline__ void shade_pixel(const DrawParams &D, const SH &S, int ti, int qx, int y, int i,
                                            float col[4], uint32_t &lvMask)
{
    // the plane record in 16-byte pieces: x0 y0 zA zB | zC wA wB wC | then A, B, C
    // of each varying from float 8
    const float4 p0 = S.planeA[ti][0], p1 = S.planeA[ti][1];
    const float x0p = p0.x, y0p = p0.y;
    const float wA = p1.y, wB = p1.z, wC = p1.w;
    const float xFi = ((float)qx + (float)(i & 1)) - x0p;
    const float yFi = ((float)y + (float)(i >> 1)) - y0p;
    const float rhwI = 1.0f / mul_add(xFi, wA, wC + yFi * wB);
    float c[4];
    {
        const float4 p2 = S.planeA[ti][2], p3 = S.planeA[ti][3], p4 = S.planeA[ti][4];
        const float cA[4] = {p2.x, p2.w, p3.z, p4.y}, cB[4] = {p2.y, p3.x, p3.w, p4.z}, cC[4] = {p2.z, p3.y, p4.x, p4.w};
#pragma unroll
        for(int k = 0; k < 4; k++) c[k] = mul_add(xFi, cA[k], cC[k] + yFi * cB[k]) * rhwI;
    }
    if(D.fs == SWGB_FS_TEX_X_VCOLOR)
    {
        const float4 p5 = S.planeA[ti][5], p6 = S.planeA[ti][6];
        const float uA = p5.x, uB = p5.y, uC = p5.z;
        const float vA = p5.w, vB = p6.x, vC = p6.y;
        float u[4], v[4];
#pragma unroll
        for(int j = 0; j < 4; j++)
        {
            if(j == 3 && i != 3) break;  // lane 3 only feeds itself
            const float xF = ((float)qx + (float)(j & 1)) - x0p;
            const float yF = ((float)y + (float)(j >> 1)) - y0p;
            const float r = j == i ? rhwI : 1.0f / mul_add(xF, wA, wC + yF * wB);
            u[j] = mul_add(xF, uA, uC + yF * uB) * r;
            v[j] = mul_add(xF, vA, vC + yF * vB) * r;
        }
        const float lod = implicit_lod(D, u, v);
        const float ul = i == 0 ? u[0] : (i == 1 ? u[1] : (i == 2 ? u[2] : u[3]));
        const float vl = i == 0 ? v[0] : (i == 1 ? v[1] : (i == 2 ? v[2] : v[3]));
        float t[4];
        if(D.floatPath)
        {
            // temporaries: t and lvMask stay in registers on the UNORM8 path
            float tf[4];
            uint32_t lm = 0u;
            sample_float_lane<SH::kFull>(D, lod, ul, vl, tf, lm);
            lvMask |= lm;
#pragma unroll
            for(int k = 0; k < 4; k++) t[k] = tf[k];
        }
        else sample_texture_lane<SH::kFull, TEXFAST>(D, lod, ul, vl, t, lvMask);
#pragma unroll
        for(int k = 0; k < 4; k++) c[k] = t[k] * c[k];
    }
#pragma unroll
    for(int k = 0; k < 4; k++) col[k] = cf_unorm8(CF) ? rmin(rmax(c[k], 0.0f), 1.0f) : c[k];  // clampColor: UNORM only
}

// Depth test/write, blend and colour write of one pixel of the staged bin
// (PixelRoutine.cpp:494-574,660-685; alphaBlend :1653-1961; writeColor
// :1975-1993,2429-2650).
template<int CF, class SH>
__device__ __forceinline__ void rop_pixel(const DrawParams &D, SH &S, int ti, int q, int idx, float z, const float col[4],
                                          unsigned long long &nTested, unsigned long long &nPassed)
{
    float *depth = S.depth[q];
    uint32_t *color = S.color[q];
    if(!SH::kFull)
    {
        if(D.depthTest)
        {
            nTested++;
            if(!depth_pass(D.compareOp, depth[idx], z)) return;
            if(D.depthWrite) depth[idx] = z;
        }
    }
    else
    {
        // masks as PixelRoutine::quad forms them (:97-124,330-358,530-575):
        // the depth and bounds tests give zMask (with a depth test) or trim
        // the coverage (without one); the stencil op then sees failOp /
        // depthFailOp / passOp; depth and colour are written where every
        // test passed
        bool zPass = true;
        if(D.depthTest)
        {
            nTested++;
            const float stored = depth[idx];
            zPass = depth_pass(D.compareOp, stored, z) && (!D.depthBounds || bounds_pass(D, stored));
        }
        else if(D.depthBounds && !bounds_pass(D, depth[idx]))
            return;  // outside the coverage: no stencil op either
        if(D.stencilTest && !stencil_resolve(D, &S.stencil[q][idx], S.front[ti] ? 0 : 1, zPass)) return;
        if(!zPass) return;
        if(D.depthWrite) depth[idx] = z;
    }
    nPassed++;
    float out[4];
    if(D.blend)
    {
        float dst[4];
        if(cf_unorm8(CF))
        {
            // readPixel widens b to b * 257, alphaBlend scales by 1 / 0xFFFF;
            // B8G8R8A8 holds R in byte 2 and B in byte 0 (PixelRoutine.cpp:1091-1108)
            const uint32_t old = CF == CF_BGRA8 ? __byte_perm(color[idx], 0u, 0x3012u) : color[idx];
#pragma unroll
            for(int c = 0; c < 4; c++) dst[c] = (float)(((old >> (8 * c)) & 0xFFu) * 257u) * (1.0f / 0xFFFF);
            if(SH::kFull && D.colorSRGB)
            {
                float v[4] = {dst[0], dst[1], dst[2], dst[3]};
                srgb_decode3(v);  // sRGBtoLinear on R, G, B (:1822-1827)
#pragma unroll
                for(int k = 0; k < 4; k++) dst[k] = v[k];
            }
        }
        else if(CF == CF_RGBA16F)
        {
            const uint32_t w0 = color[2 * idx], w1 = color[2 * idx + 1];
            dst[0] = reactor_half_to_float(w0 & 0xFFFFu);
            dst[1] = reactor_half_to_float(w0 >> 16);
            dst[2] = reactor_half_to_float(w1 & 0xFFFFu);
            dst[3] = reactor_half_to_float(w1 >> 16);
        }
        else
        {
#pragma unroll
            for(int c = 0; c < 4; c++) dst[c] = __uint_as_float(color[4 * idx + c]);
        }
        if(D.blendAlpha)
        {
            // SRC_ALPHA, ONE_MINUS_SRC_ALPHA, ADD on colour and alpha: the
            // general path's arithmetic, inline
            const float a = col[3], oma = 1.0f - col[3];
#pragma unroll
            for(int c = 0; c < 4; c++) out[c] = col[c] * a + dst[c] * oma;
        }
        else
        {
            // temporaries: col, dst and out stay in registers on the common path
            float gc[4], gd[4], go[4];
#pragma unroll
            for(int k = 0; k < 4; k++)
            {
                gc[k] = col[k];
                gd[k] = dst[k];
            }
            blend_generic(D, gc, gd, go);
#pragma unroll
            for(int k = 0; k < 4; k++) out[k] = go[k];
        }
    }
    else
    {
#pragma unroll
        for(int c = 0; c < 4; c++) out[c] = col[c];
    }
    if(cf_unorm8(CF))
    {
        // packed in R, G, B, A byte order; B8G8R8A8 swaps R and B back on the
        // way out, and its write-mask bits with them (:2138-2143); sRGB
        // attachments encode R, G, B before the clamp (:1965-1970)
        if(SH::kFull && D.colorSRGB)
        {
            float v[4] = {out[0], out[1], out[2], out[3]};
            srgb_encode3(v);
#pragma unroll
            for(int k = 0; k < 4; k++) out[k] = v[k];
        }
        // clamped to [0, 1] (a NaN to 0), v * 255 rounds to 0..255: RoundInt's
        // out-of-range value and PackUnsigned's saturation never apply
        uint32_t fresh = 0;
#pragma unroll
        for(int c = 0; c < 4; c++)
        {
            const float v = rmin(rmax(out[c], 0.0f), 1.0f);
            fresh |= (uint32_t)__float2int_rn(v * 255.0f) << (8 * c);
        }
        if(CF == CF_BGRA8) fresh = __byte_perm(fresh, 0u, 0x3012u);
        const uint32_t keep = D.writeBytes;  // bytes of the stored texel in its own order
        color[idx] = keep == 0xFFFFFFFFu ? fresh : (color[idx] & ~keep) | (fresh & keep);
    }
    else if(CF == CF_RGBA16F)
    {
        uint32_t w[2] = {color[2 * idx], color[2 * idx + 1]};
#pragma unroll
        for(int c = 0; c < 4; c++)
            if(D.writeMask & (1u << c))
            {
                const int sh = 16 * (c & 1);
                w[c >> 1] = (w[c >> 1] & ~(0xFFFFu << sh)) | (reactor_float_to_half(out[c]) << sh);
            }
        color[2 * idx] = w[0];
        color[2 * idx + 1] = w[1];
    }
    else
    {
#pragma unroll
        for(int c = 0; c < 4; c++)
            if(D.writeMask & (1u << c)) color[4 * idx + c] = __float_as_uint(out[c]);
    }
}

__device__ __forceinline__ int warp_incl_scan(int v, int lane)
{
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
    {
        int u = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if(lane >= o) v += u;
    }
    return v;
}

// One batch of nb <= 32 triangles (primitive order) against the warp's staged
// bin.  Lane j sets up triangle j; then the warp expands quad slots, masks
// coverage, rejects early on depth, and shades the live pixels one per lane;
// lanes hitting the same pixel resolve lowest lane (earliest triangle) first.
// Depth of sample q (z per sample, QuadRasterizer.cpp:131-141 and
// PixelRoutine.cpp:128-148) at lane i of the quad at (qx, y), clamped.
template<int MS, class SH>
__device__ __forceinline__ float sample_depth(const DrawParams &D, const SH &S, int ti, int qx, int y, int i, int q)
{
    const float4 p0 = S.planeA[ti][0];
    float xF = ((float)qx + (float)(i & 1)) - p0.x;
    float yF = ((float)y + (float)(i >> 1)) - p0.y;
    if(MS > 1)
    {
        yF = yF + SLY[q];
        xF = xF - SLX[q];
    }
    float z = mul_add(xF, p0.z, S.planeA[ti][1].x + yF * p0.w);
    if(SH::kFull && D.depthBias) z = z + reinterpret_cast<const float *>(S.planeA[ti])[PLANE_ZBIAS];  // PixelRoutine.cpp:141-144
    return depth_value<SH::kFull>(D, rmin(rmax(z, D.minDepthClamp), D.maxDepthClamp));  // clampDepth
}

// Hierarchical depth rejection of whole triangle-bin pairs.  Under LESS /
// LESS_OR_EQUAL (GREATER / GREATER_OR_EQUAL) the depth of a sample only moves
// down (up), so the bin's largest (smallest) depth when a batch starts bounds
// every depth the batch's fragments meet at their ordered turn.  A NaN in the
// bin counts as passing under LESS-type ops (!(NaN <= z)) and as failing under
// GREATER-type ops, so it maps to +inf for both reductions.
template<int MS, class SH>
__device__ __forceinline__ float bin_depth_bound(const SH &S, uint32_t inMask, bool lessType)
{
    const int lane = threadIdx.x & 31;
    constexpr int BW = SH::kBW, BH = SH::kBH;
    float m = lessType ? -INFINITY : INFINITY;
#pragma unroll
    for(int q = 0; q < MS; q++)
#pragma unroll
        for(int k = 0; k < BW * BH / 32; k++)
        {
            if(!(inMask >> k & 1)) continue;  // outside the scissor: never covered
            float v = S.depth[q][lane + 32 * k];
            v = v == v ? v : INFINITY;
            m = lessType ? fmaxf(m, v) : fminf(m, v);
        }
#pragma unroll
    for(int o = 16; o > 0; o >>= 1)
    {
        const float u = __shfl_xor_sync(0xFFFFFFFFu, m, o);
        m = lessType ? fmaxf(m, u) : fminf(m, u);
    }
    return m;
}

// True when every sample of triangle ti inside the bin fails the depth test
// against the bound zb.  The plane z = zC + yF*zB + xF*zA is bounded over the
// triangle's pixel box inside the bin, widened by half a pixel for the sample
// offsets; the margin 2^-20 * (|zC| + |yF*zB| + |xF*zA|) covers the rounding of
// the kernel's three-operation evaluation and of this one.  The kernel clamps
// fragment depth to [minDepthClamp, maxDepthClamp] (and a NaN to the minimum),
// so the clamp range itself is a valid bound.
template<class SH>
__device__ __forceinline__ bool hiz_rejects(const DrawParams &D, const SH &S, int ti, uint32_t t, int bx0, int by0, float zb)
{
    const short4 box = D.triBox[t];
    const float x0p = reinterpret_cast<const float *>(S.planeA[ti])[0], y0p = reinterpret_cast<const float *>(S.planeA[ti])[1];
    const float zA = reinterpret_cast<const float *>(S.planeA[ti])[2], zB = reinterpret_cast<const float *>(S.planeA[ti])[3], zC = reinterpret_cast<const float *>(S.planeA[ti])[4];
    const float xFa = ((float)max((int)box.x, bx0) - 0.5f) - x0p, xFb = ((float)min((int)box.z, bx0 + SH::kBW) - 0.5f) - x0p;
    const float yFa = ((float)max((int)box.y, by0) - 0.5f) - y0p, yFb = ((float)min((int)box.w, by0 + SH::kBH) - 0.5f) - y0p;
    const float bias = (SH::kFull && D.depthBias) ? reinterpret_cast<const float *>(S.planeA[ti])[PLANE_ZBIAS] : 0.0f;
    const float T = fabsf(zC) + fmaxf(fabsf(yFa), fabsf(yFb)) * fabsf(zB) + fmaxf(fabsf(xFa), fabsf(xFb)) * fabsf(zA) + fabsf(bias);
    const float margin = T * (1.0f / 1048576.0f) + 1e-30f;
    const uint32_t op = D.compareOp;
    if(op == SWGB_COMPARE_LESS || op == SWGB_COMPARE_LESS_OR_EQUAL)
    {
        const float xF = zA >= 0.0f ? xFa : xFb, yF = zB >= 0.0f ? yFa : yFb;
        float zlo = (((zC + yF * zB) + xF * zA) + bias) - margin;
        if(!(zlo >= D.minDepthClamp)) zlo = D.minDepthClamp;  // also NaN
        zlo = depth_value<SH::kFull>(D, fminf(zlo, D.maxDepthClamp));
        return op == SWGB_COMPARE_LESS ? zb <= zlo : zb < zlo;
    }
    const float xF = zA >= 0.0f ? xFb : xFa, yF = zB >= 0.0f ? yFb : yFa;
    float zhi = (((zC + yF * zB) + xF * zA) + bias) + margin;
    if(!(zhi <= D.maxDepthClamp)) zhi = D.maxDepthClamp;
    zhi = depth_value<SH::kFull>(D, fmaxf(zhi, D.minDepthClamp));
    return op == SWGB_COMPARE_GREATER ? zb >= zhi : zb > zhi;
}

// Covered samples and quads of triangle ti inside the bin, from its staged span
// rows: a sample of pixel x is covered iff left <= x < right, a quad counts when
// any sample of its two pixels in its two rows is covered (the counts the quad
// path makes for the same triangle).
template<int MS, class SH>
__device__ __forceinline__ void covered_counts(const SH &S, int ti, int bx0, uint32_t &samples, uint32_t &quads)
{
    samples = 0;
    quads = 0;
    const int qr0 = S.qr0[ti], nqr = S.nqr[ti];
    for(int k = 0; k < nqr; k++)
    {
        const int qr = qr0 + k;
        uint32_t colMask = 0;
#pragma unroll
        for(int q = 0; q < MS; q++)
#pragma unroll
            for(int r = 0; r < 2; r++)
            {
                const uint32_t sp = S.span[ti][q][2 * qr + r];
                const int l = max((int)(sp & 0xFFFF), bx0) - bx0, rr = min((int)(sp >> 16), bx0 + SH::kBW) - bx0;
                if(l < rr)
                {
                    samples += (uint32_t)(rr - l);
                    const int ca = l >> 1, cb = (rr - 1) >> 1;
                    colMask |= ((2u << cb) - 1u) & ~((1u << ca) - 1u);
                }
            }
        quads += __popc(colMask);
    }
}

// Whole triangles behind the bin are counted, not expanded: returns the lane's
// quad slot count, 0 when its triangle is rejected.
template<int MS, class SH>
__device__ __noinline__ int hiz_pass(const DrawParams &D, int cnt, int bx0, int by0, uint32_t inMask, bool lessType,
                                     unsigned long long &nQuads, unsigned long long &nTested)
{
    // the warp's staging block from the kernel's dynamic shared memory (as
    // k_raster lays it out), so that it is addressed as shared memory here
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const SH &S = reinterpret_cast<const SH *>(smem_raw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    if(!__any_sync(0xFFFFFFFFu, cnt > 0)) return cnt;
    const float zb = bin_depth_bound<MS>(S, inMask, lessType);
    if(cnt > 0 && hiz_rejects(D, S, lane, (uint32_t)S.triList[lane], bx0, by0, zb))
    {
        uint32_t ns, nq;
        covered_counts<MS>(S, lane, bx0, ns, nq);
        nTested += ns;
        nQuads += nq;
        cnt = 0;
    }
    return cnt;
}

// One batch of nb <= 32 triangles (primitive order) against the warp's staged
// bin.  Lane j sets up triangle j; then the warp expands quad slots, masks
// coverage per sample, rejects early on depth, and shades the live pixels one
// per lane (once per pixel, at its centre); lanes hitting the same pixel
// resolve lowest lane (earliest triangle) first, all of the pixel's samples
// at once.
template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL>
__device__ __forceinline__ void raster_batch_body(const DrawParams &D, RasterShared<CF, MS, BW, BH, FULL> &S, int nb, int bx0, int by0,
                                             uint32_t inMask, unsigned long long &nQuadsIo, unsigned long long &nTestedIo,
                                             unsigned long long &nPassedIo, uint32_t &lvMaskIo, int w0 = 0, int w1 = BH)
{
    // the counters in registers for the batch: no out-of-line call takes
    // their address, and the queue's shared-memory stores cannot alias them
    unsigned long long nQuads = nQuadsIo, nTested = nTestedIo, nPassed = nPassedIo;
    uint32_t lvMask = lvMaskIo;
    const int lane = threadIdx.x & 31;
    int cnt = 0;
    if(lane < nb) cnt = setup_batch_triangle(D, S, lane, (uint32_t)S.triList[lane], bx0, by0, w0, w1);
    __syncwarp();
    // Depth only moves one way under LESS/LESS_OR_EQUAL (down) and GREATER/
    // GREATER_OR_EQUAL (up) with clamped, never-NaN fragment depth, so a
    // sample that fails against the bin's current depth fails at its ordered
    // turn too.
    const bool lessType = D.compareOp == SWGB_COMPARE_LESS || D.compareOp == SWGB_COMPARE_LESS_OR_EQUAL;
    const bool earlyZ = D.depthTest && (!FULL || D.earlyDepthOK) &&
                        (lessType || D.compareOp == SWGB_COMPARE_GREATER || D.compareOp == SWGB_COMPARE_GREATER_OR_EQUAL);
    if(HIZ && earlyZ)
    {
        unsigned long long hq = 0ull, ht = 0ull;
        cnt = hiz_pass<MS, RasterShared<CF, MS, BW, BH, FULL>>(D, cnt, bx0, by0, inMask, lessType, hq, ht);
        nQuads += hq;
        nTested += ht;
    }
    const int incl = warp_incl_scan(cnt, lane);
    const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    // Quad rounds expand 32 quad slots each and append their live pixels to
    // the queue S.pixq; pixel rounds take 32 queued pixels at a time (the
    // rest after the last quad round).  A pixel queued but not yet resolved
    // leaves the staged depth as it was, which only makes a later quad
    // round's early test reject less.
    int qn = 0;  // queued pixels (warp-uniform)
    for(int s0 = 0;; s0 += 32)
    {
        const bool drain = s0 >= total;
        if(!drain)
        {
            // ---- quad slot -> (triangle, quad) -> coverage, early depth ---------
            const int slot = s0 + lane;
            int src;
            if constexpr(!HIZ && MS == 1 && !FULL)
            {
                // the triangle owning slot s0 + lane: each triangle with slots
                // in the window marks where they start there (distinct
                // positions: its slots are a non-empty run), and a lane takes
                // the last mark at or before its position -- one vote and one
                // shared read instead of five dependent shuffles (height field
                // 0.666 -> 0.657 ms; the rejection variants keep the search,
                // 1% faster there on the atlas)
                const int first = max(incl - cnt, s0) - s0;
                const bool in = cnt > 0 && incl - cnt < s0 + 32 && incl > s0;
                if(in) S.owner[first] = (uint8_t)lane;
                const unsigned marks = __reduce_or_sync(0xFFFFFFFFu, in ? 1u << first : 0u);
                __syncwarp();
                const unsigned m = marks & (0xFFFFFFFFu >> (31 - lane));
                src = m ? (int)S.owner[31 - __clz(m)] : 0;
            }
            else
            {
                int lo = 0, hi = 31;  // smallest lane j with incl_j > slot
#pragma unroll
                for(int step = 0; step < 5; step++)
                {
                    int mid = (lo + hi) >> 1;
                    int v = __shfl_sync(0xFFFFFFFFu, incl, mid);
                    if(v > slot) hi = mid; else lo = mid + 1;
                }
                src = lo;
            }
            const int sIncl = __shfl_sync(0xFFFFFFFFu, incl, src);
            const int sCnt = __shfl_sync(0xFFFFFFFFu, cnt, src);
            int cMask = 0, qti = src, qx = 0, qrow = 0;  // cMask bit 4q+i: sample q of lane i
            if(slot < total)
            {
                const int local = slot - (sIncl - sCnt);
                // the quad row: the rows after the first whose quad prefix is <= local
                // (the prefix never decreases), counted with independent reads
                const int nq = S.nqr[qti];
                int k = 0;
#pragma unroll
                for(int j = 1; j < BH / 2; j++) k += (j < nq && (int)S.qpre[qti][j] <= local) ? 1 : 0;
                qrow = S.qr0[qti] + k;
                qx = S.qx0[qti][k] + 2 * (local - (int)S.qpre[qti][k]);
#pragma unroll
                for(int q = 0; q < MS; q++)
                {
                    const uint32_t sp0 = S.span[qti][q][2 * qrow], sp1 = S.span[qti][q][2 * qrow + 1];
                    const int l0 = sp0 & 0xFFFF, r0 = sp0 >> 16, l1 = sp1 & 0xFFFF, r1 = sp1 >> 16;
                    // per-lane coverage: left <= x < right (QuadRasterizer.cpp:184-209)
                    int m = 0;
                    if(qx >= l0 && qx < r0) m |= 1;
                    if(qx + 1 >= l0 && qx + 1 < r0) m |= 2;
                    if(qx >= l1 && qx < r1) m |= 4;
                    if(qx + 1 >= l1 && qx + 1 < r1) m |= 8;
                    cMask |= m << (4 * q);
                }
                if(cMask)
                {
                    nQuads++;
                    if(earlyZ)
                    {
                        // the quad's depth, as sample_depth computes it, with the
                        // triangle's z plane read once: x and y relative to the
                        // plane origin per column / row, z = MulAdd(x, A, C + y B)
                        const int lx = qx - bx0, ly = 2 * qrow, y = by0 + 2 * qrow;
                        const float4 p0 = S.planeA[qti][0];
                        const float x0p = p0.x, y0p = p0.y, zA = p0.z, zB = p0.w, zC = S.planeA[qti][1].x;
                        const float zBias = (FULL && D.depthBias) ? reinterpret_cast<const float *>(S.planeA[qti])[PLANE_ZBIAS] : 0.0f;
                        const float xc[2] = {(float)qx - x0p, ((float)qx + 1.0f) - x0p};
                        const float yr[2] = {(float)y - y0p, ((float)y + 1.0f) - y0p};
                        int keep = 0;
#pragma unroll
                        for(int q = 0; q < MS; q++)
#pragma unroll
                            for(int i = 0; i < 4; i++)
                            {
                                if(!(cMask >> (4 * q + i) & 1)) continue;
                                float xF = xc[i & 1], yF = yr[i >> 1];
                                if(MS > 1)
                                {
                                    yF = yF + SLY[q];
                                    xF = xF - SLX[q];
                                }
                                float z = mul_add(xF, zA, zC + yF * zB);
                                if(FULL && D.depthBias) z = z + zBias;
                                z = depth_value<FULL>(D, rmin(rmax(z, D.minDepthClamp), D.maxDepthClamp));
                                if(depth_pass(D.compareOp, S.depth[q][(ly + (i >> 1)) * BW + lx + (i & 1)], z)) keep |= 1 << (4 * q + i);
                            }
                        nTested += __popc(cMask & ~keep);
                        cMask = keep;
                    }
                }
            }
            // ---- live pixels (any live sample) into the queue ---------------------
            int pixMask = 0;
#pragma unroll
            for(int q = 0; q < MS; q++) pixMask |= (cMask >> (4 * q)) & 0xF;
            const int np = __popc(pixMask);
            const int pIncl = warp_incl_scan(np, lane);
            int pos = qn + pIncl - np;
#pragma unroll
            for(int b = 0; b < 4; b++)
                if(pixMask >> b & 1)
                {
                    int sm = 0;  // the pixel's live samples
#pragma unroll
                    for(int q = 0; q < MS; q++) sm |= ((cMask >> (4 * q + b)) & 1) << q;
                    S.pixq[pos++] = (uint32_t)qti | (uint32_t)(qx - bx0) << 5 | (uint32_t)qrow << 11 | (uint32_t)b << 16 | (uint32_t)sm << 18;
                }
            qn += __shfl_sync(0xFFFFFFFFu, pIncl, 31);
            __syncwarp();
        }
        // ---- pixel rounds: 32 queued pixels, one per lane ---------------------
        int done = 0;
        while(qn - done >= 32 || (drain && qn > done))
        {
            const bool valid = lane < qn - done;
            int pidx = -1 - lane, i = 0, sm = 0, qTi = 0, qX = 0, qRow = 0;
            float col[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if(valid)
            {
                const uint32_t e = S.pixq[done + lane];
                qTi = (int)(e & 31u);
                qX = bx0 + (int)((e >> 5) & 63u);
                qRow = (int)((e >> 11) & 31u);
                i = (int)((e >> 16) & 3u);
                sm = (int)((e >> 18) & 15u);
                pidx = (2 * qRow + (i >> 1)) * BW + (qX - bx0) + (i & 1);
                shade_pixel<CF, !HIZ>(D, S, qTi, qX, by0 + 2 * qRow, i, col, lvMask);
            }
            // ordered resolve: among lanes on the same pixel, lowest lane first
            // (rank = earlier lanes on the lane's pixel)
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, pidx);
            const int rank = __popc(peers & ((1u << lane) - 1u));
            const int maxRank = __reduce_max_sync(0xFFFFFFFFu, (unsigned)rank);
            for(int rr = 0; rr <= maxRank; rr++)
            {
                if(valid && rank == rr)
                {
#pragma unroll
                    for(int q = 0; q < MS; q++)
                        if(sm >> q & 1)
                        {
                            const float z = D.depthTest ? sample_depth<MS>(D, S, qTi, qX, by0 + 2 * qRow, i, q) : 0.0f;
                            rop_pixel<CF>(D, S, qTi, q, pidx, z, col, nTested, nPassed);
                        }
                }
                __syncwarp();
            }
            done += min(32, qn - done);
        }
        if(drain) break;
        if(done)
        {
            // the leftover (< 32) moves to the front
            const int rem = qn - done;
            const uint32_t v = lane < rem ? S.pixq[done + lane] : 0u;
            __syncwarp();
            if(lane < rem) S.pixq[lane] = v;
            __syncwarp();
            qn = rem;
        }
    }
    nQuadsIo = nQuads;
    nTestedIo = nTested;
    nPassedIo = nPassed;
    lvMaskIo = lvMask;
    __syncwarp();
}

// raster_batch_body out of line: the variants with hierarchical depth
// rejection, four samples or the full pixel pipeline call it so (inlined into
// their kernels, the 32x16 and 16x16 rejection variants on the full atlas
// took 1343 and 1706 ms instead of 882 and 1164; this wrapper under another
// name measured 4% slower on the atlas with the same registers and stack).
// Out of line it finds the warp's staging block in the dynamic shared memory
// itself, rather than taking it as a (generic) reference: atlas 884 -> 870 ms.
// Inlined, the single-sample common variants address the staged bin as
// shared memory throughout (out of line it arrives as a generic pointer) and
// allocate their registers with the bin loop: on the 1M-triangle height
// field k_raster took 0.680 ms instead of 0.744.
template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL>
__device__ __noinline__ void raster_batch(const DrawParams &D, int nb, int bx0, int by0, uint32_t inMask, unsigned long long &nQuads,
                                          unsigned long long &nTested, unsigned long long &nPassed, uint32_t &lvMask)
{
    // the warp's staging block from the kernel's dynamic shared memory (as
    // k_raster lays it out), so that it is addressed as shared memory here
    extern __shared__ __align__(16) uint8_t smem_raw[];
    RasterShared<CF, MS, BW, BH, FULL> &S = reinterpret_cast<RasterShared<CF, MS, BW, BH, FULL> *>(smem_raw)[threadIdx.x >> 5];
    raster_batch_body<CF, MS, BW, BH, HIZ, FULL>(D, S, nb, bx0, by0, inMask, nQuads, nTested, nPassed, lvMask);
}

template<int BW, int BH>
__device__ __forceinline__ bool box_hits(short4 b, int bx0, int by0)
{
    return b.x < b.z && b.x < bx0 + BW && b.z > bx0 && b.y < by0 + BH && b.w > by0;
}

template<int BW, int BH>
__device__ __forceinline__ bool box_hits(int4 b, int bx0, int by0)
{
    return b.x < b.z && b.x < bx0 + BW && b.z > bx0 && b.y < by0 + BH && b.w > by0;
}

__device__ __forceinline__ void flush_counters(unsigned long long *counters, unsigned long long nQuads, unsigned long long nTested,
                                               unsigned long long nPassed, uint32_t lvMask)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for(int o = 16; o > 0; o >>= 1)
    {
        nQuads += __shfl_xor_sync(0xFFFFFFFFu, nQuads, o);
        nTested += __shfl_xor_sync(0xFFFFFFFFu, nTested, o);
        nPassed += __shfl_xor_sync(0xFFFFFFFFu, nPassed, o);
        lvMask |= __shfl_xor_sync(0xFFFFFFFFu, lvMask, o);
    }
    if(lane == 0 && (nQuads | nTested | nPassed | lvMask))
    {
        atomicAdd(&counters[4], nQuads);
        atomicAdd(&counters[5], nTested);
        atomicAdd(&counters[6], nPassed);
        atomicOr(&counters[7], (unsigned long long)lvMask);
    }
}

// Walks the candidates of the bin at (bx0, by0) in primitive order --
// super-chunk, chunk, then triangle boxes, compacted with ballots into
// S.triList -- and hands them to batch(nb) BATCH at a time (nb < BATCH for the
// last call).
template<class SH, class F>
__device__ __forceinline__ void walk_bin(const DrawParams &D, SH &S, int bx0, int by0, F &&batch)
{
    const int lane = threadIdx.x & 31;
    constexpr int BW = SH::kBW, BH = SH::kBH;
    int listCount = 0;  // warp-uniform
    for(int sb = 0; sb < D.nsuper; sb += 32)
    {
        unsigned superHits = __ballot_sync(0xFFFFFFFFu, sb + lane < D.nsuper && box_hits<BW, BH>(D.superBox[sb + lane], bx0, by0));
        while(superHits)
        {
            const int sc = sb + __ffs(superHits) - 1;
            superHits &= superHits - 1;
            static_assert(SUPER % 32 == 0 && CHUNK == 32, "chunk boxes in ballots of 32, one triangle per lane");
#pragma unroll
            for(int cw = 0; cw < SUPER; cw += 32)
            {
            const int c = sc * SUPER + cw + lane;
            unsigned chunkHits = __ballot_sync(0xFFFFFFFFu, c < D.nchunks && box_hits<BW, BH>(D.chunkBox[c], bx0, by0));
            while(chunkHits)
            {
                const int chunk = sc * SUPER + cw + __ffs(chunkHits) - 1;
                chunkHits &= chunkHits - 1;
                short4 tb = make_short4(0, 0, 0, 0);
                if((uint32_t)chunk * CHUNK + lane < D.count) tb = D.triBox[(uint32_t)chunk * CHUNK + lane];
                {
                    const uint32_t tri = (uint32_t)chunk * CHUNK + lane;
                    const bool th = tri < D.count && box_hits<BW, BH>(tb, bx0, by0);
                    const unsigned b = __ballot_sync(0xFFFFFFFFu, th);
                    if(th) S.triList[listCount + __popc(b & ((1u << lane) - 1u))] = (int)tri;
                    listCount += __popc(b);
                    __syncwarp();
                    if(listCount >= BATCH)
                    {
                        batch(BATCH);
                        const int rem = listCount - BATCH;
                        const int v = lane < rem ? S.triList[BATCH + lane] : 0;
                        __syncwarp();
                        if(lane < rem) S.triList[lane] = v;
                        listCount = rem;
                        __syncwarp();
                    }
                }
            }
            }
        }
    }
    if(listCount > 0) batch(listCount);
}

// One bin of a draw (part 0), or the top (1) / bottom (2) half of its rows:
// stage its depth and colour, walk the candidates in primitive order in
// batches, write the bin back.
template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL>
__device__ __forceinline__ void raster_bin(const DrawParams &D, RasterShared<CF, MS, BW, BH, FULL> &S, int bin, int part, unsigned long long &nQuads,
                                           unsigned long long &nTested, unsigned long long &nPassed, uint32_t &lvMask)
{
    const int lane = threadIdx.x & 31;
    constexpr int CW = color_words(CF);
    const int bx0 = D.binX0 + (bin % D.binsX) * BW;
    const int by0 = D.binY0 + (bin / D.binsX) * BH;
    // rows [w0, w1) of the bin: all, or the top / bottom half of a split bin
    // (the other half's warp stages and writes back its own rows)
    const int w0 = part == 2 ? BH / 2 : 0, w1 = part == 1 ? BH / 2 : BH;

    // The bin is staged when its first batch arrives: a bin no candidate
    // reaches is neither read nor written back.
    bool staged = false;
    auto stage = [&]() {
        // ---- stage the bin's depth and colour, every sample plane (16-byte segments) ----
        for(int q = 0; q < MS; q++)
        {
            const uint8_t *dbase = D.depth + (size_t)q * D.depthSlice;
            const uint8_t *cbase = D.color + (size_t)q * D.colorSlice;
            for(int i = lane; i < BW * BH / 4; i += 32)
            {
                const int ly = i / (BW / 4), lx = (i % (BW / 4)) * 4;
                if(ly < w0 || ly >= w1) continue;
                const int px = bx0 + lx, py = by0 + ly;
                float4 dz = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
                if((D.depthTest || (FULL && D.depthBounds)) && py < D.sy1 && px < D.sx1)
                {
                    const uint8_t *drow = dbase + (size_t)py * D.depthPitch;
                    if(FULL && D.depth16)
                    {
                        // D16_UNORM: the stored integers as floats (readDepth16)
                        uint32_t w0 = 0, w1 = 0;
                        if(D.vec16 && px + 4 <= D.sx1)
                        {
                            const uint2 v = *(const uint2 *)(drow + (size_t)px * 2);
                            w0 = v.x;
                            w1 = v.y;
                        }
                        else
                        {
                            uint32_t h[4] = {0, 0, 0, 0};
                            for(int k = 0; k < 4 && px + k < D.sx1; k++) h[k] = *(const uint16_t *)(drow + (size_t)(px + k) * 2);
                            w0 = h[0] | h[1] << 16;
                            w1 = h[2] | h[3] << 16;
                        }
                        dz = make_float4((float)(w0 & 0xFFFFu), (float)(w0 >> 16), (float)(w1 & 0xFFFFu), (float)(w1 >> 16));
                    }
                    else if(D.vec16 && px + 4 <= D.sx1)
                        dz = *(const float4 *)(drow + (size_t)px * 4);
                    else
                    {
                        float dv[4] = {1.0f, 1.0f, 1.0f, 1.0f};
                        for(int k = 0; k < 4 && px + k < D.sx1; k++) dv[k] = *(const float *)(drow + (size_t)(px + k) * 4);
                        dz = make_float4(dv[0], dv[1], dv[2], dv[3]);
                    }
                }
                *(float4 *)&S.depth[q][ly * BW + lx] = dz;
            }
            for(int i = lane; i < BW * BH * CW / 4; i += 32)
            {
                // 16-byte segment i of the bin's colour rows: 4 / CW pixels
                const int ly = i / (BW * CW / 4), lx = (i % (BW * CW / 4)) * 4 / CW;
                if(ly < w0 || ly >= w1) continue;
                const int px = bx0 + lx, py = by0 + ly;
                uint4 cc = make_uint4(0, 0, 0, 0);
                if(py < D.sy1 && px < D.sx1)
                {
                    const uint8_t *crow = cbase + (size_t)py * D.colorPitch + (size_t)px * 4 * CW;
                    if(D.vec16 && px + 4 / CW <= D.sx1)
                        cc = *(const uint4 *)crow;
                    else
                    {
                        uint32_t cv[4] = {0, 0, 0, 0};
                        for(int k = 0; k < 4 && px + k / CW < D.sx1; k++) cv[k] = *(const uint32_t *)(crow + 4 * k);
                        cc = make_uint4(cv[0], cv[1], cv[2], cv[3]);
                    }
                }
                *(uint4 *)&S.color[q][(ly * BW + lx) * CW] = cc;
            }
        }
        if(FULL && D.stencilTest)
            for(int q = 0; q < MS; q++)
            {
                // the bin's stencil bytes (1 per pixel and sample plane)
                const uint8_t *sbase = D.stencil + (size_t)q * D.stencilSlice;
                for(int i = lane; i < BW * BH; i += 32)
                {
                    const int px = bx0 + i % BW, py = by0 + i / BW;
                    S.stencil[q][i] = (py < D.sy1 && px < D.sx1) ? sbase[(size_t)py * D.stencilPitch + px] : (uint8_t)0;
                }
            }
        __syncwarp();
    };

    // bit k: pixel lane + 32k of the bin lies inside the scissor (the depth bound's domain)
    uint32_t inMask = 0;
    if(HIZ)
#pragma unroll
        for(int k = 0; k < BW * BH / 32; k++)
        {
            const int idx = lane + 32 * k;
            const int px = bx0 + (idx % BW), py = by0 + idx / BW;
            if(px >= D.sx0 && px < D.sx1 && py >= D.sy0 && py < D.sy1) inMask |= 1u << k;
        }

    // ---- candidates in primitive order, in batches of BATCH ----------------------
    auto batch = [&](int nb) {
        if(!staged)
        {
            stage();
            staged = true;
        }
        if constexpr(!HIZ && MS == 1 && !FULL)
            raster_batch_body<CF, MS, BW, BH, HIZ, FULL>(D, S, nb, bx0, by0, inMask, nQuads, nTested, nPassed, lvMask, w0, w1);
        else
            raster_batch<CF, MS, BW, BH, HIZ, FULL>(D, nb, bx0, by0, inMask, nQuads, nTested, nPassed, lvMask);
    };
    const uint32_t listed = D.binList ? __ldg(D.binListCount + bin) : 0xFFFFFFFFu;
    if(listed <= D.binListCap)
    {
        // the bin's list from k_bin_list
        const uint32_t *list = D.binList + (size_t)bin * D.binListCap;
        for(uint32_t i = 0; i < listed; i += BATCH)
        {
            const int nb = (int)min((uint32_t)BATCH, listed - i);
            if(lane < nb) S.triList[lane] = (int)__ldg(list + i + lane);
            __syncwarp();
            batch(nb);
        }
    }
    else
        walk_bin(D, S, bx0, by0, batch);
    if(!staged) return;  // untouched bin

    // ---- write the bin back, every sample plane ----------------------------------
    if(FULL && D.stencilWrite)
        for(int q = 0; q < MS; q++)
        {
            uint8_t *sbase = D.stencil + (size_t)q * D.stencilSlice;
            for(int i = lane; i < BW * BH; i += 32)
            {
                const int px = bx0 + i % BW, py = by0 + i / BW;
                if(py >= D.sy0 && py < D.sy1 && px >= D.sx0 && px < D.sx1 && i / BW >= w0 && i / BW < w1)
                    sbase[(size_t)py * D.stencilPitch + px] = S.stencil[q][i];
            }
        }
    for(int q = 0; q < MS; q++)
    {
        uint8_t *dbase = D.depth + (size_t)q * D.depthSlice;
        uint8_t *cbase = D.color + (size_t)q * D.colorSlice;
        for(int i = lane; i < BW * BH / 4; i += 32)
        {
            if(!D.depthWrite) break;
            const int ly = i / (BW / 4), lx = (i % (BW / 4)) * 4;
            const int px = bx0 + lx, py = by0 + ly;
            if(py >= D.sy1 || px >= D.sx1 || py < D.sy0 || ly < w0 || ly >= w1) continue;
            uint8_t *drow = dbase + (size_t)py * D.depthPitch;
            if(FULL && D.depth16)
            {
                // D16_UNORM: the staged values are integers 0..65535
                const float4 v = *(const float4 *)&S.depth[q][ly * BW + lx];
                const uint32_t h[4] = {(uint32_t)v.x, (uint32_t)v.y, (uint32_t)v.z, (uint32_t)v.w};
                if(D.vec16 && px + 4 <= D.sx1 && px >= D.sx0)
                    *(uint2 *)(drow + (size_t)px * 2) = make_uint2(h[0] | h[1] << 16, h[2] | h[3] << 16);
                else
                    for(int k = 0; k < 4 && px + k < D.sx1; k++)
                        if(px + k >= D.sx0) *(uint16_t *)(drow + (size_t)(px + k) * 2) = (uint16_t)h[k];
            }
            else if(D.vec16 && px + 4 <= D.sx1 && px >= D.sx0)
                *(float4 *)(drow + (size_t)px * 4) = *(const float4 *)&S.depth[q][ly * BW + lx];
            else
                for(int k = 0; k < 4 && px + k < D.sx1; k++)
                    if(px + k >= D.sx0) *(float *)(drow + (size_t)(px + k) * 4) = S.depth[q][ly * BW + lx + k];
        }
        for(int i = lane; i < BW * BH * CW / 4; i += 32)
        {
            const int ly = i / (BW * CW / 4), lx = (i % (BW * CW / 4)) * 4 / CW;
            const int px = bx0 + lx, py = by0 + ly;
            if(py >= D.sy1 || px >= D.sx1 || py < D.sy0 || ly < w0 || ly >= w1) continue;
            uint8_t *crow = cbase + (size_t)py * D.colorPitch + (size_t)px * 4 * CW;
            if(D.vec16 && px + 4 / CW <= D.sx1 && px >= D.sx0)
                *(uint4 *)crow = *(const uint4 *)&S.color[q][(ly * BW + lx) * CW];
            else
                for(int k = 0; k < 4 && px + k / CW < D.sx1; k++)
                    if(px + k / CW >= D.sx0) *(uint32_t *)(crow + 4 * k) = S.color[q][(ly * BW + lx) * CW + k];
        }
    }
    __syncwarp();
}

// Shared memory of a raster block and the blocks one SM holds with it, at
// most 5 for the single-sample variants of the common pixel pipeline and
// those with hierarchical depth rejection, 4 for the rest: the register
// budget follows from that (65536 / (blocks x threads): 102 and 128
// registers).  Measured on the 1M-triangle frame (no rejection): with the
// batch loop out of line, 4 blocks 0.954 ms against 1.010 for 5 (96
// registers) and 0.952 for 3; with it inlined (92 registers at 5 blocks, no
// spills) 5 blocks 0.662 ms against 0.681 for 4 and 0.675 for 3.  On the full
// atlas's 16x16 rejection variant 5 blocks 1150 ms against 1172 for 4 and
// 1345 for 3; a 6-block bound (80 registers, spilling) lost 5% earlier.
template<int CF, int MS, int BW, int BH, bool FULL>
constexpr size_t raster_smem()
{
    static_assert(sizeof(RasterShared<CF, MS, BW, BH, FULL>) % 16 == 0, "each warp's shared block starts 16-byte aligned");
    return RASTER_WARPS * sizeof(RasterShared<CF, MS, BW, BH, FULL>);
}
template<int CF, int MS, int BW, int BH, bool FULL, bool HIZ = false>
constexpr int raster_min_blocks()
{
    return (int)std::min<size_t>(HIZ || (MS == 1 && !FULL) ? 5 : 4,
                                 std::max<size_t>(1, (size_t)(228 * 1024) / (raster_smem<CF, MS, BW, BH, FULL>() + 1024)));
}

template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL>
__global__ void __launch_bounds__(RASTER_THREADS, (raster_min_blocks<CF, MS, BW, BH, FULL, HIZ>())) k_raster(const __grid_constant__ DrawParams D)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    RasterShared<CF, MS, BW, BH, FULL> &S = reinterpret_cast<RasterShared<CF, MS, BW, BH, FULL> *>(smem_raw)[warp];
    const int nbins = D.binsX * D.binsY;
    // queue entries: the bins, or with an order its entries (split bins twice)
    const int entries = D.binOrder ? (int)__ldg(D.binOrder + 2 * nbins) : nbins;
    unsigned long long nQuads = 0, nTested = 0, nPassed = 0;
    uint32_t lvMask = 0;
    // Persistent warps: each takes the next queue entry (a bin, or half of a
    // split one) until the queue drains, so a slow bin never holds idle warps
    // of its block.
    for(;;)
    {
        int item = 0;
        if(lane == 0) item = (int)atomicAdd(D.binQueue, 1u);
        item = __shfl_sync(0xFFFFFFFFu, item, 0);
        if(item >= entries) break;
        const uint32_t e = D.binOrder ? __ldg(D.binOrder + item) : (uint32_t)item;
        raster_bin<CF, MS, BW, BH, HIZ, FULL>(D, S, (int)(e & 0x3FFFFFFFu), (int)(e >> 30), nQuads, nTested, nPassed, lvMask);
    }
    flush_counters(D.counters, nQuads, nTested, nPassed, lvMask);
}

// ------------------------------------------------------------------------
// Batched draws: N independent draws in one launch of each kernel.  Work units
// (vertex blocks, setup blocks, bins) of all draws form one index space; a
// unit finds its draw by binary search over the per-draw prefix arrays.  The
// grids are persistent (grid-stride / atomic queue), and all counts live in
// device memory, so one captured graph serves any batch shape.
// ------------------------------------------------------------------------

struct BatchHeader {
    uint32_t n;        // draws
    uint32_t vblocks;  // vertex blocks (256 vertices each)
    uint32_t sblocks;  // setup blocks (256 triangles each)
    uint32_t bins;     // bins
    uint32_t nsuper;   // super-chunk boxes of all draws
    // byte offsets from the header of the draw records and of the three
    // n + 1 prefix arrays; they depend on n, so they travel with the data and
    // a captured graph serves any n
    uint32_t offDraws, offV, offS, offB;
    uint32_t offAdj;  // per-draw AdjParams (adjoint batches only)
    uint32_t split;   // adjoint batches: warps per bin (1 or 4)
    uint32_t pad[5];
};

struct BatchPtrs {
    const BatchHeader *hdr;
    int4 *superAll;
    unsigned int *binQueue;
    uint32_t *polyCount;
    unsigned long long *spanCount;
    unsigned long long *counters;
};

// The header and the arrays it locates.
struct BatchView {
    BatchHeader h;
    const DrawParams *draws;
    const uint32_t *vStart, *sStart, *bStart;
    __device__ __forceinline__ explicit BatchView(const BatchHeader *p) : h(*p)
    {
        const uint8_t *base = (const uint8_t *)p;
        draws = (const DrawParams *)(base + h.offDraws);
        vStart = (const uint32_t *)(base + h.offV);
        sStart = (const uint32_t *)(base + h.offS);
        bStart = (const uint32_t *)(base + h.offB);
    }
};

// Largest d < n with start[d] <= u (start is non-decreasing, start[0] = 0).
__device__ __forceinline__ uint32_t find_draw(const uint32_t *start, uint32_t n, uint32_t u)
{
    uint32_t lo = 0, hi = n - 1;
    while(lo < hi)
    {
        uint32_t mid = (lo + hi + 1) >> 1;
        if(__ldg(start + mid) <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
}

#ifndef SWGB_RASTER_TU
__global__ void __launch_bounds__(256) k_vertex_batch(const __grid_constant__ BatchPtrs B)
{
    const BatchView V(B.hdr);
    const BatchHeader &h = V.h;
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    if(gtid == 0)
    {
        *B.polyCount = 0;
        *B.spanCount = 0;
        *B.binQueue = 0;
    }
    for(uint32_t j = gtid; j < h.nsuper; j += gridDim.x * blockDim.x)
        B.superAll[j] = make_int4(0x7FFFFFFF, 0x7FFFFFFF, (int)0x80000000, (int)0x80000000);
    for(uint32_t u = blockIdx.x; u < h.vblocks; u += gridDim.x)
    {
        const uint32_t d = find_draw(V.vStart, h.n, u);
        const DrawParams &D = V.draws[d];
        const uint32_t i = (u - __ldg(V.vStart + d)) * 256 + threadIdx.x;
        if(i < D.vertexCount) vertex_body(D, i);
    }
}

__global__ void __launch_bounds__(SETUP_THREADS, 3) k_setup_batch(const __grid_constant__ BatchPtrs B)
{
    const BatchView V(B.hdr);
    const BatchHeader &h = V.h;
    for(uint32_t u = blockIdx.x; u < h.sblocks; u += gridDim.x)
    {
        const uint32_t d = find_draw(V.sStart, h.n, u);
        setup_body<false>(V.draws[d], u - __ldg(V.sStart + d));
    }
}

#endif  // SWGB_RASTER_TU

template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL>
__global__ void __launch_bounds__(RASTER_THREADS, (raster_min_blocks<CF, MS, BW, BH, FULL, HIZ>())) k_raster_batch(const __grid_constant__ BatchPtrs B)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    RasterShared<CF, MS, BW, BH, FULL> &S = reinterpret_cast<RasterShared<CF, MS, BW, BH, FULL> *>(smem_raw)[warp];
    const BatchView V(B.hdr);
    const BatchHeader &h = V.h;
    unsigned long long nQuads = 0, nTested = 0, nPassed = 0;
    uint32_t lvMask = 0;
    for(;;)
    {
        uint32_t bin = 0;
        if(lane == 0) bin = atomicAdd(B.binQueue, 1u);
        bin = __shfl_sync(0xFFFFFFFFu, bin, 0);
        if(bin >= h.bins) break;
        const uint32_t d = find_draw(V.bStart, h.n, bin);
        raster_bin<CF, MS, BW, BH, HIZ, FULL>(V.draws[d], S, (int)(bin - __ldg(V.bStart + d)), 0, nQuads, nTested, nPassed, lvMask);
    }
    flush_counters(B.counters, nQuads, nTested, nPassed, lvMask);
}

#ifndef SWGB_RASTER_TU
#include "swgb_adjoint.cuh"
#endif


// ------------------------------------------------------------------------
// Raster kernel variants: bin shape x depth rejection x colour format x
// samples.  The instantiations live in swgb_raster.cu (one object per colour
// format); fill_raster_table<CF> fills the table entries of format CF.
// ------------------------------------------------------------------------
struct RasterKernel {
    const void *fn;       // k_raster instantiation
    const void *fnBatch;  // k_raster_batch instantiation
    size_t smem;          // dynamic shared memory per block
    void (*launch)(const DrawParams &, uint32_t, cudaStream_t);
    void (*launchBatch)(const BatchPtrs &, uint32_t, cudaStream_t);
};

// Table index of a variant: single-sample draws by (shape, hiz, format);
// four-sample draws (16x16) by (hiz, format); draws needing the full
// per-sample pipeline (16x16) by (samples, hiz, format).
__host__ __device__ constexpr int raster_index(int shape, bool hiz, int ms, int cf, bool full)
{
    return full ? NSHAPES * 2 * NCF + 2 * NCF + ((ms > 1 ? 2 : 0) + (hiz ? 0 : 1)) * NCF + cf
               : (ms > 1 ? NSHAPES * 2 * NCF + (hiz ? 0 : 1) * NCF + cf : (shape * 2 + (hiz ? 0 : 1)) * NCF + cf);
}

template<int CF>
void fill_raster_table(RasterKernel *table);
template<> void fill_raster_table<CF_RGBA8>(RasterKernel *table);
template<> void fill_raster_table<CF_RGBA16F>(RasterKernel *table);
template<> void fill_raster_table<CF_RGBA32F>(RasterKernel *table);
template<> void fill_raster_table<CF_BGRA8>(RasterKernel *table);

}  // namespace swgbk

#endif  // SWGB_KERNELS_CUH
