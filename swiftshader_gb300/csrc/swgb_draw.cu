// swgb_draw.cu -- GB300 (sm_103a) kernels and C-ABI of the draw hot path.
//
// Pipeline per draw (all on the context's stream, no host round trip):
//   k_vertex  : one thread per vertex -- fetch, fixed VS (MVP), clip flags,
//               projection + viewport snap.  Post-transform vertices stay in
//               HBM/L2 like the reference's vertex cache
//               (src/Pipeline/VertexRoutine.cpp:43-87,116-154,570-707).
//   k_setup   : one thread per triangle, 256-triangle chunks -- trivial
//               reject, homogeneous clipping, cull, sub-pixel polygon, y range,
//               empty-row trimming, pixel bounding box; block-reduced chunk
//               boxes drive the binning (src/Device/Renderer.cpp:733-776,
//               src/Device/Clipper.cpp, src/Pipeline/SetupRoutine.cpp:36-294).
//   k_raster  : one CTA per 32x32-pixel bin -- depth and colour of the bin are
//               staged in shared memory; the chunk boxes and triangle boxes are
//               tested in primitive order (warp ballot + prefix compaction);
//               each batch of triangles regenerates its span rows with the
//               reference's integer DDA, expands into 2x2 quad fragments,
//               shades them in parallel (interpolation, SamplerCore filtering,
//               fixed FS), and resolves depth test + blend per quad in
//               primitive order; the bin is written back with 128-bit stores
//               (src/Device/QuadRasterizer.cpp:36-250,
//               src/Pipeline/PixelRoutine.cpp:97-358,494-739,1225-2700,
//               src/Pipeline/PixelProgram.cpp:138-364,
//               src/Pipeline/SamplerCore.cpp).
#include <cuda_runtime.h>
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

#include "../../include/swgb.h"
#include "swgb_numeric.cuh"

using namespace swgb;

namespace {

constexpr int MAXV = 7;          // varying components carried per vertex
constexpr int BIN = 16;          // bin side in pixels; one warp owns one bin
constexpr int RASTER_WARPS = 4;  // independent warps (bins) per raster block
constexpr int RASTER_THREADS = 32 * RASTER_WARPS;
constexpr int BATCH = 32;        // triangles staged per batch: one per lane
constexpr int SUPER = 32;        // chunks per super-chunk box
constexpr int SETUP_THREADS = 256;
constexpr int CHUNK = 64;        // triangles per chunk box
constexpr int MAX_POLY = 16;     // clipped polygon capacity (Polygon::B, src/Device/Polygon.hpp:45)

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
    uint32_t info;     // bits 0-4: polygon vertex count, bit 5: winding d, bit 6: clipped, bit 7: spans stored
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
    float minDepthClamp, maxDepthClamp;
    int blend;
    uint32_t srcC, dstC, opC, srcA, dstA, opA;
    uint32_t writeMask;
    int fs;
    int ms;       // samples per pixel: 1 or 4
    uint64_t colorSlice, depthSlice;  // bytes between sample planes
    int cf;       // colour attachment format, CF_*
    int texFloat; // 0: R8G8B8A8_UNORM texture (16-bit path), 1: RGBA16F, 2: RGBA32F (fp32 path)
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
    uint32_t addrU, addrV;
    // bins
    int binX0, binY0, binsX, binsY;
    int nchunks;
    // scratch
    float4 *ptv;          // 4 x float4 per vertex
    double *ptv64;        // adjoint runs only: clip x, y, w and x/w, y/w in fp64 (6 doubles per vertex), else null
    short4 *triBox;       // pixel box per triangle
    TriInfo *triInfo;
    short4 *chunkBox;     // union of the boxes of CHUNK consecutive triangles
    int4 *superBox;       // union of SUPER consecutive chunk boxes (x0, y0, x1, y1)
    int nsuper;
    unsigned int *binQueue;  // next bin for the persistent raster warps
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
    if(i < nverts) vertex_body(D, i);
}

// ------------------------------------------------------------------------
// Setup stage
// ------------------------------------------------------------------------

__device__ __forceinline__ uint32_t fetch_index(const DrawParams &D, uint32_t k)
{
    if(D.indexType == SWGB_INDEX_TYPE_NONE) return k;
    if(D.indexType == SWGB_INDEX_TYPE_UINT16) return __ldg((const uint16_t *)D.indices + k);
    if(D.indexType == SWGB_INDEX_TYPE_UINT8) return __ldg((const uint8_t *)D.indices + k);
    return __ldg((const uint32_t *)D.indices + k);
}

// Post-transform vertex slots of triangle t: the index-buffer positions of
// setBatchIndices with the first vertex provoking (Renderer.cpp:97-134) --
// list (3t, 3t+1, 3t+2); strip (t, t+1+odd, t+2-odd), odd = t & 1; fan
// (t+1, t+2, 0) -- through the index buffer of an indexed draw.
__device__ __forceinline__ void tri_slots(const DrawParams &D, uint32_t t, uint32_t &i0, uint32_t &i1, uint32_t &i2)
{
    uint32_t k0, k1, k2;
    if(D.topology == SWGB_TOPOLOGY_TRIANGLE_STRIP)
    {
        k0 = t;
        k1 = t + 1 + (t & 1);
        k2 = t + 2 - (t & 1);
    }
    else if(D.topology == SWGB_TOPOLOGY_TRIANGLE_FAN)
    {
        k0 = t + 1;
        k1 = t + 2;
        k2 = 0;
    }
    else
    {
        k0 = 3 * t;
        k1 = 3 * t + 1;
        k2 = 3 * t + 2;
    }
    i0 = fetch_index(D, k0);
    i1 = fetch_index(D, k1);
    i2 = fetch_index(D, k2);
}

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
__device__ int clip_polygon(CVert *P, int n, int flagsOr)
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
__device__ void span_at(const DrawParams &D, const int32_t *X, const int32_t *Y, int n, int dW, int32_t y, int32_t &l, int32_t &r)
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
__device__ void write_spans(const DrawParams &D, const int32_t *X, const int32_t *Y, int n, int dW, int32_t yMin, uint32_t *sp)
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
__device__ __forceinline__ void setup_body(const DrawParams &D, uint32_t blk)
{
    const uint32_t t = blk * SETUP_THREADS + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    short4 box = make_short4(0, 0, 0, 0);
    TriInfo inf = {0u, 0u, 0u, 0u};
    int cntIn = 0, cntClip = 0, cntVis = 0;
    bool cand = false;
    int n = 3, dW = 1;
    int32_t X[MAX_POLY + 1], Y[MAX_POLY + 1];
    int32_t yMin = 0, yMax = 0, xMinS = 0, xMaxS = 0;
    if(t < D.count)
    {
        cntIn = 1;
        uint32_t i0, i1, i2;
        bool ok = true;
        tri_slots(D, t, i0, i1, i2);
        if(D.indexType != SWGB_INDEX_TYPE_NONE && (i0 >= D.vertexCount || i1 >= D.vertexCount || i2 >= D.vertexCount))
        {
            atomicOr(D.error, ERR_INDEX_RANGE);
            ok = false;
        }
        if(ok)
        {
            const float4 p0 = D.ptv[(size_t)i0 * 4 + 1], p1 = D.ptv[(size_t)i1 * 4 + 1], p2 = D.ptv[(size_t)i2 * 4 + 1];
            const int f0 = __float_as_int(p0.z), f1 = __float_as_int(p1.z), f2 = __float_as_int(p2.z);
            X[0] = __float_as_int(p0.x); X[1] = __float_as_int(p1.x); X[2] = __float_as_int(p2.x);
            Y[0] = __float_as_int(p0.y); Y[1] = __float_as_int(p1.y); Y[2] = __float_as_int(p2.y);
            // setupSolidTriangles trivial reject (src/Device/Renderer.cpp:749-765)
            if((f0 & f1 & f2) == CLIP_FINITE)
            {
                const float4 c0 = D.ptv[(size_t)i0 * 4], c1 = D.ptv[(size_t)i1 * 4], c2 = D.ptv[(size_t)i2 * 4];
                const int flagsOr = f0 | f1 | f2;
                bool keep = true;
                CVert P[MAX_POLY];
                if(flagsOr != CLIP_FINITE)
                {
                    cntClip = 1;
                    P[0] = {c0.x, c0.y, c0.z, c0.w};
                    P[1] = {c1.x, c1.y, c1.z, c1.w};
                    P[2] = {c2.x, c2.y, c2.z, c2.w};
                    n = clip_polygon(P, 3, flagsOr);
                    keep = n >= 3;
                }
                if(keep)
                {
                    // Culling (SetupRoutine.cpp:73-120)
                    float x0 = (float)X[0], x1 = (float)X[1], x2 = (float)X[2];
                    float y0 = (float)Y[0], y1 = (float)Y[1], y2 = (float)Y[2];
                    float A = ((y0 - y2) * x1 + (y2 - y1) * x0) + (y1 - y0) * x2;
                    int32_t w0w1w2 = __float_as_int(c0.w) ^ __float_as_int(c1.w) ^ __float_as_int(c2.w);
                    if(w0w1w2 < 0) A = -A;
                    bool front = D.frontFace == SWGB_FRONT_FACE_COUNTER_CLOCKWISE ? (A >= 0.0f) : (A <= 0.0f);
                    if((D.cullMode & SWGB_CULL_FRONT) && front) keep = false;
                    if((D.cullMode & SWGB_CULL_BACK) && !front) keep = false;
                    dW = A > 0.0f ? 1 : 0;
                }
                if(keep && cntClip)
                {
                    // reproject the clipped polygon (SetupRoutine.cpp:125-145)
                    for(int i = 0; i < n; i++)
                    {
                        float w = P[i].w;
                        float rhw = w != 0.0f ? 1.0f / w : 1.0f;
                        X[i] = round_int(D.X0xF + (P[i].x * rhw) * D.WxF);
                        Y[i] = round_int(D.Y0xF + (P[i].y * rhw) * D.HxF);
                    }
                }
                if(keep)
                {
                    yMin = Y[0]; yMax = Y[0]; xMinS = X[0]; xMaxS = X[0];
                    for(int i = 1; i < n; i++)
                    {
                        yMin = min(yMin, Y[i]); yMax = max(yMax, Y[i]);
                        xMinS = min(xMinS, X[i]); xMaxS = max(xMaxS, X[i]);
                    }
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

    // ---- allocate span rows: block scan + one atomic per block ----------
    __shared__ uint32_t sWarp[SETUP_THREADS / 32];
    __shared__ unsigned long long sBase;
    const uint32_t rows = cand ? (uint32_t)(yMax - yMin) : 0u;
    uint32_t incl = rows * (uint32_t)D.ms;
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
    {
        uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if(lane >= o) incl += u;
    }
    if(lane == 31) sWarp[warp] = incl;
    __syncthreads();
    if(threadIdx.x == 0)
    {
        uint32_t tot = 0;
        for(int w = 0; w < SETUP_THREADS / 32; w++)
        {
            uint32_t c = sWarp[w];
            sWarp[w] = tot;
            tot += c;
        }
        sBase = tot ? atomicAdd(D.spanCount, (unsigned long long)tot) : 0ull;
    }
    __syncthreads();
    const uint64_t off = (uint64_t)sBase + sWarp[warp] + (incl - rows * (uint32_t)D.ms);

    bool stored = false;
    if(cand && D.ms > 1)
    {
        // 4x MSAA: one outline per sample, the polygon shifted by -Xf/-Yf
        // (SetupRoutine.cpp:188-240); rows no edge writes stay empty and
        // nothing is trimmed.
        stored = off + (uint64_t)rows * 4 <= (uint64_t)D.spanCapacity;
        if(stored)
        {
            for(int q = 0; q < 4; q++)
            {
                uint32_t *sp = D.spans + off + (uint64_t)q * rows;
                for(uint32_t r = 0; r < rows; r++) sp[r] = 0u;
                int32_t Xq[MAX_POLY + 1], Yq[MAX_POLY + 1];
                for(int i = 0; i < n; i++) { Xq[i] = X[i] - XF[q]; Yq[i] = Y[i] - YF[q]; }
                write_spans(D, Xq, Yq, n, dW, yMin, sp);
            }
            inf.spanOff = (uint32_t)off;
            inf.rows = rows;
        }
    }
    else if(cand)
    {
        stored = off + rows <= (uint64_t)D.spanCapacity;
        if(stored)
        {
            uint32_t *sp = D.spans + off;
            write_spans(D, X, Y, n, dW, yMin, sp);
            // Trim empty rows at the top and bottom (SetupRoutine.cpp:243-264)
            const int32_t y0 = yMin;
            while(yMin < yMax)
            {
                uint32_t s = sp[yMin - y0];
                if((s & 0xFFFFu) != (s >> 16)) break;
                yMin++;
            }
            while(yMax > yMin)
            {
                uint32_t s = sp[yMax - 1 - y0];
                if((s & 0xFFFFu) != (s >> 16)) break;
                yMax--;
            }
            inf.spanOff = (uint32_t)(off + (uint64_t)(yMin - y0));
        }
        else
        {
            // span scratch full: trim by direct evaluation; k_raster walks the
            // edges itself for this triangle
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
    }
    if(cand && yMin < yMax)
    {
        {
            // pixel box: covered x satisfy ceil(Xmin/256) <= left <= x < right <= ceil(Xmax/256)
            const int32_t pad = D.ms > 1 ? 96 : 0;  // farthest sample offset (Xf)
            int32_t bx0 = max(D.sx0, (xMinS - pad + 0xFF) >> 8);
            int32_t bx1 = max(bx0, min(D.sx1, (xMaxS + pad + 0xFF) >> 8));
            {
                cntVis = 1;
                box = make_short4((short)bx0, (short)yMin, (short)bx1, (short)yMax);
                inf.info = (uint32_t)n | ((uint32_t)dW << 5) | ((uint32_t)cntClip << 6) | ((uint32_t)stored << 7);
                if(!stored) inf.rows = 0;
                if(cntClip)
                {
                    uint32_t slot = atomicAdd(D.polyCount, 1u);
                    if(slot < D.polyCapacity)
                    {
                        inf.slot = slot;
                        for(int i = 0; i < n; i++) D.poly[(size_t)slot * MAX_POLY + i] = make_int2(X[i], Y[i]);
                    }
                    else
                    {
                        atomicOr(D.error, ERR_POLY_OVERFLOW);
                        cntVis = 0;
                        box = make_short4(0, 0, 0, 0);
                        inf.info = 0;
                    }
                }
            }
        }
    }
    D.triBox[t] = box;  // capacity is a whole number of setup blocks
    D.triInfo[t] = inf;

    // ---- chunk boxes (64 triangles = 2 warps) and counters ------------------
    const bool has = cntVis != 0;
    int bx0 = has ? box.x : 0x7FFF, by0 = has ? box.y : 0x7FFF;
    int bx1 = has ? box.z : -0x8000, by1 = has ? box.w : -0x8000;
    int cntRej = cntIn - cntVis;
#pragma unroll
    for(int o = 16; o > 0; o >>= 1)
    {
        bx0 = min(bx0, __shfl_xor_sync(0xFFFFFFFFu, bx0, o));
        by0 = min(by0, __shfl_xor_sync(0xFFFFFFFFu, by0, o));
        bx1 = max(bx1, __shfl_xor_sync(0xFFFFFFFFu, bx1, o));
        by1 = max(by1, __shfl_xor_sync(0xFFFFFFFFu, by1, o));
        cntIn += __shfl_xor_sync(0xFFFFFFFFu, cntIn, o);
        cntRej += __shfl_xor_sync(0xFFFFFFFFu, cntRej, o);
        cntClip += __shfl_xor_sync(0xFFFFFFFFu, cntClip, o);
        cntVis += __shfl_xor_sync(0xFFFFFFFFu, cntVis, o);
    }
    __shared__ short4 sBox[SETUP_THREADS / 32];
    __shared__ int sCnt[4][SETUP_THREADS / 32];
    if(lane == 0)
    {
        sBox[warp] = make_short4((short)bx0, (short)by0, (short)bx1, (short)by1);
        sCnt[0][warp] = cntIn; sCnt[1][warp] = cntRej; sCnt[2][warp] = cntClip; sCnt[3][warp] = cntVis;
    }
    __syncthreads();
    if(threadIdx.x < SETUP_THREADS / CHUNK)
    {
        const int w0 = threadIdx.x * (CHUNK / 32);
        short4 b = sBox[w0];
        for(int w = 1; w < CHUNK / 32; w++)
        {
            short4 c = sBox[w0 + w];
            b.x = min(b.x, c.x); b.y = min(b.y, c.y); b.z = max(b.z, c.z); b.w = max(b.w, c.w);
        }
        D.chunkBox[blk * (SETUP_THREADS / CHUNK) + threadIdx.x] = b;
        if(b.x < b.z)
        {
            int4 *sb = D.superBox + blk / (SUPER * CHUNK / SETUP_THREADS);
            atomicMin(&sb->x, (int)b.x);
            atomicMin(&sb->y, (int)b.y);
            atomicMax(&sb->z, (int)b.z);
            atomicMax(&sb->w, (int)b.w);
        }
    }
    if(threadIdx.x == 0)
    {
        int a = 0, b = 0, c = 0, d = 0;
        for(int w = 0; w < SETUP_THREADS / 32; w++) { a += sCnt[0][w]; b += sCnt[1][w]; c += sCnt[2][w]; d += sCnt[3][w]; }
        atomicAdd(&D.counters[0], (unsigned long long)a);
        atomicAdd(&D.counters[1], (unsigned long long)b);
        atomicAdd(&D.counters[2], (unsigned long long)c);
        atomicAdd(&D.counters[3], (unsigned long long)d);
    }
}

__global__ void __launch_bounds__(SETUP_THREADS) k_setup(const __grid_constant__ DrawParams D) { setup_body(D, blockIdx.x); }

// ------------------------------------------------------------------------
// SamplerCore 16-bit path for R8G8B8A8_UNORM (src/Pipeline/SamplerCore.cpp)
// ------------------------------------------------------------------------

// address() 16-bit (SamplerCore.cpp:2399-2435)
__device__ __forceinline__ uint32_t address16(float uw, uint32_t mode)
{
    if(mode == SWGB_ADDRESS_CLAMP_TO_EDGE)
    {
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
__device__ __forceinline__ uint32_t texel_rgba8(const TexLevel &lv, uint32_t u, uint32_t v)
{
    uint32_t xi = mulhi_u16(u, lv.w);
    uint32_t yi = mulhi_u16(v, lv.h);
    int32_t index = (int32_t)(int16_t)xi + (int32_t)(int16_t)yi * (int32_t)(int16_t)lv.pitch;  // pmaddwd
    return __ldg((const uint32_t *)lv.buf + (uint32_t)index);
}

// sampleQuad2D for one lane, 16-bit channel values c << 8 (SamplerCore.cpp:668-909).
__device__ __forceinline__ void sample_quad_2d(const DrawParams &D, float u, float v, float lod, int second, uint32_t out[4], uint32_t &lvMask)
{
    int ilod = D.mipLinear ? trunc_int(lod) : round_int(lod);  // selectMipmap (:2357-2379)
    int li = ilod + second;
    li = li < 0 ? 0 : (li > D.levelCount - 1 ? D.levelCount - 1 : li);
    lvMask |= 1u << li;
    const TexLevel &lv = D.lv[li];
    uint32_t uu = address16(u, D.addrU);
    uint32_t vv = address16(v, D.addrV);
    if(!D.texLinear)
    {
        uint32_t t = texel_rgba8(lv, uu, vv);
#pragma unroll
        for(int c = 0; c < 4; c++) out[c] = ((t >> (8 * c)) & 0xFFu) << 8;
        return;
    }
    bool wu = D.addrU == SWGB_ADDRESS_REPEAT, wv = D.addrV == SWGB_ADDRESS_REPEAT;
    uint32_t u0 = offset_sample(uu, lv.uHalf, wu, -1), v0 = offset_sample(vv, lv.vHalf, wv, -1);
    uint32_t u1 = offset_sample(uu, lv.uHalf, wu, +1), v1 = offset_sample(vv, lv.vHalf, wv, +1);
    uint32_t t00 = texel_rgba8(lv, u0, v0), t10 = texel_rgba8(lv, u1, v0);
    uint32_t t01 = texel_rgba8(lv, u0, v1), t11 = texel_rgba8(lv, u1, v1);
    // bilinearInterpolate, unsigned 8-bit components (:516-575)
    uint32_t f0u = (u0 * lv.w) & 0xFFFFu, f0v = (v0 * lv.h) & 0xFFFFu;
    uint32_t f1u = (~f0u) & 0xFFFFu, f1v = (~f0v) & 0xFFFFu;
    uint32_t f0u0v = mulhi_u16(f0u, f0v), f1u0v = mulhi_u16(f1u, f0v);
    uint32_t f0u1v = mulhi_u16(f0u, f1v), f1u1v = mulhi_u16(f1u, f1v);
#pragma unroll
    for(int c = 0; c < 4; c++)
    {
        uint32_t a = mulhi_u16(((t00 >> (8 * c)) & 0xFFu) << 8, f1u1v);
        uint32_t b = mulhi_u16(((t10 >> (8 * c)) & 0xFFu) << 8, f0u1v);
        uint32_t e = mulhi_u16(((t01 >> (8 * c)) & 0xFFu) << 8, f1u0v);
        uint32_t g = mulhi_u16(((t11 >> (8 * c)) & 0xFFu) << 8, f0u0v);
        out[c] = (((a + b) & 0xFFFFu) + ((e + g) & 0xFFFFu)) & 0xFFFFu;
    }
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
__device__ __forceinline__ void sample_texture_lane(const DrawParams &D, float lod, float ul, float vl, float out[4],
                                                    uint32_t &lvMask)
{
    uint32_t c[4], cc[4] = {0u, 0u, 0u, 0u};
    const int levels = D.mipLinear ? 2 : 1;
#pragma unroll 1
    for(int second = 0; second < levels; second++)
    {
        uint32_t t[4];
        sample_quad_2d(D, ul, vl, lod, second, t, lvMask);
#pragma unroll
        for(int k = 0; k < 4; k++)
        {
            if(second) cc[k] = t[k]; else c[k] = t[k];
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
    else
        coord = rmin(coord - floorf(coord), one);  // Float4 Frac (LLVMReactor.cpp:3252-3275)
    coord = coord * (float)dim;
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
    if(D.texFloat == 2) return __ldg((const float4 *)lv.buf + (uint32_t)index);
    const uint2 h = __ldg((const uint2 *)lv.buf + (uint32_t)index);
    return make_float4(half_bits_to_float(h.x & 0xFFFFu), half_bits_to_float(h.x >> 16),
                       half_bits_to_float(h.y & 0xFFFFu), half_bits_to_float(h.y >> 16));
}

// sampleFloat2D for one lane (SamplerCore.cpp:1155-1248).
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
__device__ __forceinline__ void sample_float_lane(const DrawParams &D, float lod, float ul, float vl, float out[4], uint32_t &lvMask)
{
    float4 c = sample_float_2d(D, ul, vl, lod, 0, lvMask);
    if(D.mipLinear)
    {
        const float4 cc = sample_float_2d(D, ul, vl, lod, 1, lvMask);
        const float fr = lod - floorf(lod);
        c.x = (cc.x - c.x) * fr + c.x;
        c.y = (cc.y - c.y) * fr + c.y;
        c.z = (cc.z - c.z) * fr + c.z;
        c.w = (cc.w - c.w) * fr + c.w;
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
constexpr int PLANE_V = 6;  // varying components with plane equations (colour + uv)
constexpr int PLANES = 8 + 3 * PLANE_V;

// 32-bit words per pixel of a colour attachment: R8G8B8A8_UNORM,
// R16G16B16A16_SFLOAT, R32G32B32A32_SFLOAT.
enum { CF_RGBA8 = 0, CF_RGBA16F = 1, CF_RGBA32F = 2 };
__host__ __device__ constexpr int color_words(int cf) { return cf == CF_RGBA8 ? 1 : (cf == CF_RGBA16F ? 2 : 4); }

// Shared memory of one warp: its bin's depth and colour, the staged batch,
// and its ordered candidate list.
template<int CF, int MS>
struct RasterShared {
    float depth[MS][BIN * BIN];
    uint32_t color[MS][BIN * BIN * color_words(CF)];
    float plane[PLANES][BATCH];
    uint32_t span[BATCH][MS][BIN];      // left | right << 16 per sample and bin row
    int16_t qx0[BATCH][BIN / 2];        // first quad x per quad row of the triangle
    uint16_t qpre[BATCH][BIN / 2 + 1];  // prefix of quads per quad row
    int8_t qr0[BATCH];                  // first quad row of the triangle in the bin
    int8_t nqr[BATCH];                  // quad rows of the triangle in the bin
    int triList[2 * BATCH];
    static constexpr int kSamples = MS;
};

__device__ __forceinline__ uint32_t select3(int o, uint32_t a, uint32_t b, uint32_t c) { return o == 0 ? a : (o == 1 ? b : c); }

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

// R1: one batch triangle -- its span rows inside the bin (from the setup
// stage's span buffer, or the reference DDA when the buffer was full), its
// quad rows, and its plane equations (SetupRoutine.cpp:270-548).  Returns the
// number of quad slots it expands to.
template<class SH>
__device__ int setup_batch_triangle(const DrawParams &D, SH &S, int ti, uint32_t t, int bx0, int by0)
{
    const short4 box = D.triBox[t];
    const TriInfo inf = D.triInfo[t];
    const int n = inf.info & 31, dW = (inf.info >> 5) & 1;
    const int rowLo = max((int)box.y, by0), rowHi = min((int)box.w, by0 + BIN);  // bin rows of the triangle
    const int qrA = (rowLo - by0) >> 1, qrB = (rowHi - 1 - by0) >> 1;            // quad rows [qrA, qrB]
    constexpr int MS = SH::kSamples;
    // rows outside [rowLo, rowHi) but inside the quad rows are empty
#pragma unroll
    for(int q = 0; q < MS; q++)
    {
        S.span[ti][q][2 * qrA] = 0u;
        S.span[ti][q][2 * qrB + 1] = 0u;
    }
    if(inf.info & 128)
    {
#pragma unroll
        for(int q = 0; q < MS; q++)
        {
            const uint32_t *sp = D.spans + inf.spanOff + (size_t)q * inf.rows + (rowLo - box.y);
            for(int y = rowLo; y < rowHi; y++) S.span[ti][q][y - by0] = __ldg(sp + (y - rowLo));
        }
    }
    else
    {
        // span scratch was full at setup: walk the edges here (SetupRoutine::edge)
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
            xb = min(xb, bx0 + BIN);
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

    // plane equations from the post-transform vertices (L2 resident)
    uint32_t i0, i1, i2;
    tri_slots(D, t, i0, i1, i2);
    const float4 c0 = D.ptv[(size_t)i0 * 4], c1 = D.ptv[(size_t)i1 * 4], c2 = D.ptv[(size_t)i2 * 4];
    // sort by minimum y, then maximum w (SetupRoutine.cpp:270-294)
    int o0 = 0, o1 = 1, o2 = 2, tt;
    {
        float ym = rmin(rmin(c0.y, c1.y), c2.y);
        if(ym == c1.y) { tt = o0; o0 = o1; o1 = o2; o2 = tt; }
        if(ym == c2.y) { tt = o2; o2 = o1; o1 = o0; o0 = tt; }
    }
    const float cw0 = c0.w, cw1 = c1.w, cw2 = c2.w;
    {
        float w0 = o0 == 0 ? cw0 : (o0 == 1 ? cw1 : cw2);
        float w1 = o1 == 0 ? cw0 : (o1 == 1 ? cw1 : cw2);
        float w2 = o2 == 0 ? cw0 : (o2 == 1 ? cw1 : cw2);
        float wm = rmax(rmax(w0, w1), w2);
        if(wm == w1) { tt = o0; o0 = o1; o1 = o2; o2 = tt; }
        if(wm == w2) { tt = o2; o2 = o1; o1 = o0; o0 = tt; }
    }
    const uint32_t j0 = select3(o0, i0, i1, i2), j1 = select3(o1, i0, i1, i2), j2 = select3(o2, i0, i1, i2);
    const float w1 = o1 == 0 ? cw0 : (o1 == 1 ? cw1 : cw2);
    const float w2 = o2 == 0 ? cw0 : (o2 == 1 ? cw1 : cw2);
    const float4 P0 = D.ptv[(size_t)j0 * 4 + 1], P1 = D.ptv[(size_t)j1 * 4 + 1], P2 = D.ptv[(size_t)j2 * 4 + 1];
    const float4 A0 = D.ptv[(size_t)j0 * 4 + 2], A1 = D.ptv[(size_t)j1 * 4 + 2], A2 = D.ptv[(size_t)j2 * 4 + 2];
    const float rhw0 = A0.x;
    int32_t X0 = __float_as_int(P0.x), X1 = __float_as_int(P1.x), X2 = __float_as_int(P2.x);
    int32_t Y0 = __float_as_int(P0.y), Y1 = __float_as_int(P1.y), Y2 = __float_as_int(P2.y);
    const float inv = 1.0f / 256.0f;
    S.plane[0][ti] = (float)X0 * inv;
    S.plane[1][ti] = (float)Y0 * inv;
    X1 -= X0; Y1 -= Y0; X2 -= X0; Y2 -= Y0;
    float x1 = (w1 * inv) * (float)X1, y1 = (w1 * inv) * (float)Y1;
    float x2 = (w2 * inv) * (float)X2, y2 = (w2 * inv) * (float)Y2;
    float a = x1 * y2 - x2 * y1;
    float M0x = 0.0f, M0y = 0.0f, M1x = 0.0f, M1y = 0.0f, M2x = 0.0f, M2y = 0.0f;
    const float M0z = rhw0, M1z = 0.0f, M2z = 0.0f;
    if(a != 0.0f)
    {
        float A = 1.0f / a;
        float Dd = A * rhw0;
        M0x = (y1 * w2 - y2 * w1) * Dd;
        M0y = (x2 * w1 - x1 * w2) * Dd;
        M1x = y2 * A;
        M1y = (-x2) * A;
        M2x = (-y1) * A;
        M2y = x1 * A;
    }
    S.plane[5][ti] = (M0x + M1x) + M2x;
    S.plane[6][ti] = (M0y + M1y) + M2y;
    S.plane[7][ti] = (M0z + M1z) + M2z;
    if(D.depthTest)
    {
        float z0 = P0.w, z1 = P1.w - z0, z2 = P2.w - z0;
        float fx1 = (float)X1 * inv, fy1 = (float)Y1 * inv;
        float fx2 = (float)X2 * inv, fy2 = (float)Y2 * inv;
        float Dz = D.depthRange / (fx1 * fy2 - fx2 * fy1);
        S.plane[2][ti] = (fy2 * z1 - fy1 * z2) * Dz;
        S.plane[3][ti] = (fx1 * z2 - fx2 * z1) * Dz;
        S.plane[4][ti] = z0 * D.depthRange + D.depthNear;
    }
    float4 B0 = make_float4(0, 0, 0, 0), B1 = B0, B2 = B0;
    if(D.nv > 3)
    {
        B0 = D.ptv[(size_t)j0 * 4 + 3]; B1 = D.ptv[(size_t)j1 * 4 + 3]; B2 = D.ptv[(size_t)j2 * 4 + 3];
    }
#pragma unroll
    for(int k = 0; k < PLANE_V; k++)
    {
        if(k >= D.nv) break;
        float v0 = vary(A0, B0, k), v1 = vary(A1, B1, k), v2 = vary(A2, B2, k);
        S.plane[8 + 3 * k + 0][ti] = (v0 * M0x + v1 * M1x) + v2 * M2x;
        S.plane[8 + 3 * k + 1][ti] = (v0 * M0y + v1 * M1y) + v2 * M2y;
        S.plane[8 + 3 * k + 2][ti] = (v0 * M0z + v1 * M1z) + v2 * M2z;
    }
    return pre;
}

template<class SH>
__device__ __forceinline__ void quad_depth(const DrawParams &D, const SH &S, int ti, int qx, int y, float zq[4])
{
    const float x0p = S.plane[0][ti], y0p = S.plane[1][ti];
    const float zA = S.plane[2][ti], zB = S.plane[3][ti], zC = S.plane[4][ti];
#pragma unroll
    for(int i = 0; i < 4; i++)
    {
        float xF = ((float)qx + (float)(i & 1)) - x0p;
        float yF = ((float)y + (float)(i >> 1)) - y0p;
        float z = mul_add(xF, zA, zC + yF * zB);
        zq[i] = rmin(rmax(z, D.minDepthClamp), D.maxDepthClamp);  // clampDepth
    }
}

// Shades one covered pixel (lane i of the 2x2 quad at (qx, y)) of batch
// triangle ti: interpolation (PixelRoutine::quad :124-261), the fixed fragment
// shader with SamplerCore filtering (the LOD comes from lanes 0, 1 and 2 of the
// quad, covered or not, as the reference's 4-wide SIMD computes it), and the
// UNORM clamp (PixelProgram::clampColor).
template<int CF, class SH>
__device__ __forceinline__ void shade_pixel(const DrawParams &D, const SH &S, int ti, int qx, int y, int i,
                                            float col[4], uint32_t &lvMask)
{
    const float x0p = S.plane[0][ti], y0p = S.plane[1][ti];
    const float wA = S.plane[5][ti], wB = S.plane[6][ti], wC = S.plane[7][ti];
    const float xFi = ((float)qx + (float)(i & 1)) - x0p;
    const float yFi = ((float)y + (float)(i >> 1)) - y0p;
    const float rhwI = 1.0f / mul_add(xFi, wA, wC + yFi * wB);
    float c[4];
#pragma unroll
    for(int k = 0; k < 4; k++)
    {
        const float A = S.plane[8 + 3 * k][ti], B = S.plane[9 + 3 * k][ti], C = S.plane[10 + 3 * k][ti];
        c[k] = mul_add(xFi, A, C + yFi * B) * rhwI;
    }
    if(D.fs == SWGB_FS_TEX_X_VCOLOR)
    {
        const float uA = S.plane[20][ti], uB = S.plane[21][ti], uC = S.plane[22][ti];
        const float vA = S.plane[23][ti], vB = S.plane[24][ti], vC = S.plane[25][ti];
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
        if(D.texFloat) sample_float_lane(D, lod, ul, vl, t, lvMask);
        else sample_texture_lane(D, lod, ul, vl, t, lvMask);
#pragma unroll
        for(int k = 0; k < 4; k++) c[k] = t[k] * c[k];
    }
#pragma unroll
    for(int k = 0; k < 4; k++) col[k] = CF == CF_RGBA8 ? rmin(rmax(c[k], 0.0f), 1.0f) : c[k];  // clampColor: UNORM only
}

// Depth test/write, blend and colour write of one pixel of the staged bin
// (PixelRoutine.cpp:494-574,660-685; alphaBlend :1653-1961; writeColor
// :1975-1993,2429-2650).
template<int CF, int MS>
__device__ __forceinline__ void rop_pixel(const DrawParams &D, RasterShared<CF, MS> &S, int q, int idx, float z, const float col[4],
                                          unsigned long long &nTested, unsigned long long &nPassed)
{
    float *depth = S.depth[q];
    uint32_t *color = S.color[q];
    if(D.depthTest)
    {
        nTested++;
        if(!depth_pass(D.compareOp, depth[idx], z)) return;
        if(D.depthWrite) depth[idx] = z;
    }
    nPassed++;
    float out[4];
    if(D.blend)
    {
        float dst[4];
        if(CF == CF_RGBA8)
        {
            // readPixel widens b to b * 257, alphaBlend scales by 1 / 0xFFFF
            const uint32_t old = color[idx];
#pragma unroll
            for(int c = 0; c < 4; c++) dst[c] = (float)(((old >> (8 * c)) & 0xFFu) * 257u) * (1.0f / 0xFFFF);
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
    else
    {
#pragma unroll
        for(int c = 0; c < 4; c++) out[c] = col[c];
    }
    if(CF == CF_RGBA8)
    {
        uint32_t packed = color[idx];
#pragma unroll
        for(int c = 0; c < 4; c++)
        {
            float v = rmin(rmax(out[c], 0.0f), 1.0f);
            int32_t r = round_int(v * 255.0f);
            int32_t s16 = (int32_t)(int16_t)r;
            uint32_t b = s16 < 0 ? 0u : (s16 > 255 ? 255u : (uint32_t)s16);  // PackUnsigned
            if(D.writeMask & (1u << c)) packed = (packed & ~(0xFFu << (8 * c))) | (b << (8 * c));
        }
        color[idx] = packed;
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
    float xF = ((float)qx + (float)(i & 1)) - S.plane[0][ti];
    float yF = ((float)y + (float)(i >> 1)) - S.plane[1][ti];
    if(MS > 1)
    {
        yF = yF + SLY[q];
        xF = xF - SLX[q];
    }
    const float z = mul_add(xF, S.plane[2][ti], S.plane[4][ti] + yF * S.plane[3][ti]);
    return rmin(rmax(z, D.minDepthClamp), D.maxDepthClamp);  // clampDepth
}

// One batch of nb <= 32 triangles (primitive order) against the warp's staged
// bin.  Lane j sets up triangle j; then the warp expands quad slots, masks
// coverage per sample, rejects early on depth, and shades the live pixels one
// per lane (once per pixel, at its centre); lanes hitting the same pixel
// resolve lowest lane (earliest triangle) first, all of the pixel's samples
// at once.
template<int CF, int MS>
__device__ __noinline__ void raster_batch(const DrawParams &D, RasterShared<CF, MS> &S, int nb, int bx0, int by0,
                                          unsigned long long &nQuads, unsigned long long &nTested,
                                          unsigned long long &nPassed, uint32_t &lvMask)
{
    const int lane = threadIdx.x & 31;
    int cnt = 0;
    if(lane < nb) cnt = setup_batch_triangle(D, S, lane, (uint32_t)S.triList[lane], bx0, by0);
    __syncwarp();
    // Depth only moves one way under LESS/LESS_OR_EQUAL (down) and GREATER/
    // GREATER_OR_EQUAL (up) with clamped, never-NaN fragment depth, so a
    // sample that fails against the bin's current depth fails at its ordered
    // turn too.
    const bool earlyZ = D.depthTest && (D.compareOp == SWGB_COMPARE_LESS || D.compareOp == SWGB_COMPARE_LESS_OR_EQUAL ||
                                        D.compareOp == SWGB_COMPARE_GREATER || D.compareOp == SWGB_COMPARE_GREATER_OR_EQUAL);
    const int incl = warp_incl_scan(cnt, lane);
    const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    for(int s0 = 0; s0 < total; s0 += 32)
    {
        // ---- quad slot -> (triangle, quad) -> coverage, early depth ---------
        const int slot = s0 + lane;
        int src;
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
            int k = 0;
            const int nq = S.nqr[qti];
            while(k < nq - 1 && (int)S.qpre[qti][k + 1] <= local) k++;
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
                    const int lx = qx - bx0, ly = 2 * qrow, y = by0 + 2 * qrow;
                    int keep = 0;
#pragma unroll
                    for(int q = 0; q < MS; q++)
#pragma unroll
                        for(int i = 0; i < 4; i++)
                            if((cMask >> (4 * q + i) & 1) &&
                               depth_pass(D.compareOp, S.depth[q][(ly + (i >> 1)) * BIN + lx + (i & 1)], sample_depth<MS>(D, S, qti, qx, y, i, q)))
                                keep |= 1 << (4 * q + i);
                    nTested += __popc(cMask & ~keep);
                    cMask = keep;
                }
            }
        }
        // ---- live pixels (any live sample), one per lane ----------------------
        int pixMask = 0;
#pragma unroll
        for(int q = 0; q < MS; q++) pixMask |= (cMask >> (4 * q)) & 0xF;
        const int np = __popc(pixMask);
        const int pIncl = warp_incl_scan(np, lane);
        const int pTotal = __shfl_sync(0xFFFFFFFFu, pIncl, 31);
        for(int p0 = 0; p0 < pTotal; p0 += 32)
        {
            const int pix = p0 + lane;
            int lo = 0, hi = 31;
#pragma unroll
            for(int step = 0; step < 5; step++)
            {
                int mid = (lo + hi) >> 1;
                int v = __shfl_sync(0xFFFFFFFFu, pIncl, mid);
                if(v > pix) hi = mid; else lo = mid + 1;
            }
            const int qq = lo;
            const int qIncl = __shfl_sync(0xFFFFFFFFu, pIncl, qq);
            const int qN = __shfl_sync(0xFFFFFFFFu, np, qq);
            const int qPix = __shfl_sync(0xFFFFFFFFu, pixMask, qq);
            const int qMask = __shfl_sync(0xFFFFFFFFu, cMask, qq);
            const int qTi = __shfl_sync(0xFFFFFFFFu, qti, qq);
            const int qX = __shfl_sync(0xFFFFFFFFu, qx, qq);
            const int qRow = __shfl_sync(0xFFFFFFFFu, qrow, qq);
            const bool valid = pix < pTotal;
            int pidx = -1 - lane, i = 0;
            float col[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if(valid)
            {
                int nth = pix - (qIncl - qN);  // the nth set bit of the quad's pixel mask
#pragma unroll
                for(int b = 0; b < 4; b++)
                {
                    if(qPix >> b & 1)
                    {
                        if(nth == 0) i = b;
                        nth--;
                    }
                }
                pidx = (2 * qRow + (i >> 1)) * BIN + (qX - bx0) + (i & 1);
                shade_pixel<CF>(D, S, qTi, qX, by0 + 2 * qRow, i, col, lvMask);
            }
            // ordered resolve: among lanes on the same pixel, lowest lane first
            unsigned pend = __ballot_sync(0xFFFFFFFFu, valid);
            while(pend)
            {
                const bool mine = (pend >> lane) & 1;
                const unsigned peers = __match_any_sync(0xFFFFFFFFu, mine ? pidx : -1 - lane);
                if(mine && (__ffs(peers) - 1) == lane)
                {
#pragma unroll
                    for(int q = 0; q < MS; q++)
                        if(qMask >> (4 * q + i) & 1)
                        {
                            const float z = D.depthTest ? sample_depth<MS>(D, S, qTi, qX, by0 + 2 * qRow, i, q) : 0.0f;
                            rop_pixel<CF, MS>(D, S, q, pidx, z, col, nTested, nPassed);
                        }
                    pend &= ~(1u << lane);
                }
                __syncwarp();
                pend = __ballot_sync(0xFFFFFFFFu, mine && ((pend >> lane) & 1));
            }
        }
    }
    __syncwarp();
}

__device__ __forceinline__ bool box_hits(short4 b, int bx0, int by0)
{
    return b.x < b.z && b.x < bx0 + BIN && b.z > bx0 && b.y < by0 + BIN && b.w > by0;
}

__device__ __forceinline__ bool box_hits(int4 b, int bx0, int by0)
{
    return b.x < b.z && b.x < bx0 + BIN && b.z > bx0 && b.y < by0 + BIN && b.w > by0;
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
    int listCount = 0;  // warp-uniform
    for(int sb = 0; sb < D.nsuper; sb += 32)
    {
        unsigned superHits = __ballot_sync(0xFFFFFFFFu, sb + lane < D.nsuper && box_hits(D.superBox[sb + lane], bx0, by0));
        while(superHits)
        {
            const int sc = sb + __ffs(superHits) - 1;
            superHits &= superHits - 1;
            const int c = sc * SUPER + lane;
            unsigned chunkHits = __ballot_sync(0xFFFFFFFFu, c < D.nchunks && box_hits(D.chunkBox[c], bx0, by0));
            while(chunkHits)
            {
                const int chunk = sc * SUPER + __ffs(chunkHits) - 1;
                chunkHits &= chunkHits - 1;
#pragma unroll
                for(int half = 0; half < CHUNK / 32; half++)
                {
                    const uint32_t tri = (uint32_t)chunk * CHUNK + half * 32 + lane;
                    const bool th = tri < D.count && box_hits(D.triBox[tri], bx0, by0);
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
    if(listCount > 0) batch(listCount);
}

// One bin of a draw: stage its depth and colour, walk the candidates in
// primitive order in batches, write the bin back.
template<int CF, int MS>
__device__ __forceinline__ void raster_bin(const DrawParams &D, RasterShared<CF, MS> &S, int bin, unsigned long long &nQuads,
                                           unsigned long long &nTested, unsigned long long &nPassed, uint32_t &lvMask)
{
    const int lane = threadIdx.x & 31;
    constexpr int CW = color_words(CF);
    const int bx0 = D.binX0 + (bin % D.binsX) * BIN;
    const int by0 = D.binY0 + (bin / D.binsX) * BIN;

    // ---- stage the bin's depth and colour, every sample plane (16-byte segments) ----
    for(int q = 0; q < MS; q++)
    {
        const uint8_t *dbase = D.depth + (size_t)q * D.depthSlice;
        const uint8_t *cbase = D.color + (size_t)q * D.colorSlice;
        for(int i = lane; i < BIN * BIN / 4; i += 32)
        {
            const int ly = i / (BIN / 4), lx = (i % (BIN / 4)) * 4;
            const int px = bx0 + lx, py = by0 + ly;
            float4 dz = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
            if(D.depthTest && py < D.sy1 && px < D.sx1)
            {
                const uint8_t *drow = dbase + (size_t)py * D.depthPitch;
                if(D.vec16 && px + 4 <= D.sx1)
                    dz = *(const float4 *)(drow + (size_t)px * 4);
                else
                {
                    float dv[4] = {1.0f, 1.0f, 1.0f, 1.0f};
                    for(int k = 0; k < 4 && px + k < D.sx1; k++) dv[k] = *(const float *)(drow + (size_t)(px + k) * 4);
                    dz = make_float4(dv[0], dv[1], dv[2], dv[3]);
                }
            }
            *(float4 *)&S.depth[q][ly * BIN + lx] = dz;
        }
        for(int i = lane; i < BIN * BIN * CW / 4; i += 32)
        {
            // 16-byte segment i of the bin's colour rows: 4 / CW pixels
            const int ly = i / (BIN * CW / 4), lx = (i % (BIN * CW / 4)) * 4 / CW;
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
            *(uint4 *)&S.color[q][(ly * BIN + lx) * CW] = cc;
        }
    }
    __syncwarp();

    // ---- candidates in primitive order, in batches of BATCH ----------------------
    walk_bin(D, S, bx0, by0, [&](int nb) { raster_batch<CF, MS>(D, S, nb, bx0, by0, nQuads, nTested, nPassed, lvMask); });

    // ---- write the bin back, every sample plane ----------------------------------
    for(int q = 0; q < MS; q++)
    {
        uint8_t *dbase = D.depth + (size_t)q * D.depthSlice;
        uint8_t *cbase = D.color + (size_t)q * D.colorSlice;
        for(int i = lane; i < BIN * BIN / 4; i += 32)
        {
            if(!D.depthWrite) break;
            const int ly = i / (BIN / 4), lx = (i % (BIN / 4)) * 4;
            const int px = bx0 + lx, py = by0 + ly;
            if(py >= D.sy1 || px >= D.sx1 || py < D.sy0) continue;
            uint8_t *drow = dbase + (size_t)py * D.depthPitch;
            if(D.vec16 && px + 4 <= D.sx1 && px >= D.sx0)
                *(float4 *)(drow + (size_t)px * 4) = *(const float4 *)&S.depth[q][ly * BIN + lx];
            else
                for(int k = 0; k < 4 && px + k < D.sx1; k++)
                    if(px + k >= D.sx0) *(float *)(drow + (size_t)(px + k) * 4) = S.depth[q][ly * BIN + lx + k];
        }
        for(int i = lane; i < BIN * BIN * CW / 4; i += 32)
        {
            const int ly = i / (BIN * CW / 4), lx = (i % (BIN * CW / 4)) * 4 / CW;
            const int px = bx0 + lx, py = by0 + ly;
            if(py >= D.sy1 || px >= D.sx1 || py < D.sy0) continue;
            uint8_t *crow = cbase + (size_t)py * D.colorPitch + (size_t)px * 4 * CW;
            if(D.vec16 && px + 4 / CW <= D.sx1 && px >= D.sx0)
                *(uint4 *)crow = *(const uint4 *)&S.color[q][(ly * BIN + lx) * CW];
            else
                for(int k = 0; k < 4 && px + k / CW < D.sx1; k++)
                    if(px + k / CW >= D.sx0) *(uint32_t *)(crow + 4 * k) = S.color[q][(ly * BIN + lx) * CW + k];
        }
    }
    __syncwarp();
}

template<int CF, int MS>
__global__ void __launch_bounds__(RASTER_THREADS) k_raster(const __grid_constant__ DrawParams D)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    RasterShared<CF, MS> &S = reinterpret_cast<RasterShared<CF, MS> *>(smem_raw)[warp];
    const int nbins = D.binsX * D.binsY;
    unsigned long long nQuads = 0, nTested = 0, nPassed = 0;
    uint32_t lvMask = 0;
    // Persistent warps: each takes the next bin from the queue until it drains,
    // so a slow bin never holds idle warps of its block.
    for(;;)
    {
        int bin = 0;
        if(lane == 0) bin = (int)atomicAdd(D.binQueue, 1u);
        bin = __shfl_sync(0xFFFFFFFFu, bin, 0);
        if(bin >= nbins) break;
        raster_bin<CF, MS>(D, S, bin, nQuads, nTested, nPassed, lvMask);
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

__global__ void __launch_bounds__(SETUP_THREADS) k_setup_batch(const __grid_constant__ BatchPtrs B)
{
    const BatchView V(B.hdr);
    const BatchHeader &h = V.h;
    for(uint32_t u = blockIdx.x; u < h.sblocks; u += gridDim.x)
    {
        const uint32_t d = find_draw(V.sStart, h.n, u);
        setup_body(V.draws[d], u - __ldg(V.sStart + d));
        __syncthreads();  // the next unit reuses the block's shared memory
    }
}

template<int CF, int MS>
__global__ void __launch_bounds__(RASTER_THREADS) k_raster_batch(const __grid_constant__ BatchPtrs B)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    RasterShared<CF, MS> &S = reinterpret_cast<RasterShared<CF, MS> *>(smem_raw)[warp];
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
        raster_bin<CF, MS>(V.draws[d], S, (int)(bin - __ldg(V.bStart + d)), nQuads, nTested, nPassed, lvMask);
    }
    flush_counters(B.counters, nQuads, nTested, nPassed, lvMask);
}

#include "swgb_adjoint.cuh"

}  // namespace

// ==========================================================================
// Host side: context, state baking, C-ABI
// ==========================================================================

struct swgb_ctx {
    int device;
    cudaStream_t stream;
    bool ownStream;
    float4 *ptv;
    size_t ptvCap;
    short4 *triBox;
    size_t triBoxCap;
    TriInfo *triInfo;
    size_t triInfoCap;
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
    int rasterBlocks[6];  // persistent raster grid per kernel variant: SMs x resident blocks per SM
    unsigned long long *counters;
    int *error;
    uint64_t launches;
    bool rasterAttr;
    bool timing;
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
    if(st->depth_clamp_enable || st->depth_bias_constant != 0.0f || st->depth_bias_slope != 0.0f) return set_error(SWGB_UNSUPPORTED_STATE, "depth clamp / bias");
    if(st->color_format != SWGB_FORMAT_R8G8B8A8_UNORM && st->color_format != SWGB_FORMAT_R16G16B16A16_SFLOAT &&
       st->color_format != SWGB_FORMAT_R32G32B32A32_SFLOAT)
        return set_error(SWGB_UNSUPPORTED_STATE, "color_format");
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
    if(D.nattr < 2 || D.vcomp[1] != 4) return set_error(SWGB_INVALID_ARG, "the fixed FS reads a vec4 colour at location 0");
    D.fs = (int)st->fragment_shader;
    if(D.fs == SWGB_FS_TEX_X_VCOLOR && (D.nattr < 3 || D.nv < 6)) return set_error(SWGB_INVALID_ARG, "textured FS needs a uv varying");
    memcpy(D.mvp, st->mvp, sizeof(D.mvp));

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
    D.compareOp = st->depth_compare_op;
    D.minDepthClamp = 0.0f;  // no VK_EXT_depth_range_unrestricted: clamp to [0,1] (PixelProcessor.cpp:106-128)
    D.maxDepthClamp = 1.0f;
    uint32_t opC = simplify_op(st->color_blend_op, st->src_color_factor, st->dst_color_factor);
    uint32_t opA = simplify_op(st->alpha_blend_op, st->src_alpha_factor, st->dst_alpha_factor);
    D.blend = st->blend_enable && (opC != OP_SRC_EXT || opA != OP_SRC_EXT) && st->color_write_mask != 0;
    D.srcC = st->src_color_factor; D.dstC = st->dst_color_factor; D.opC = opC;
    D.srcA = st->src_alpha_factor; D.dstA = st->dst_alpha_factor; D.opA = opA;
    D.writeMask = st->color_write_mask & 0xFu;
    D.ms = (int)st->sample_count;
    D.colorSlice = st->color_slice_bytes;
    D.depthSlice = st->depth_slice_bytes;
    D.cf = st->color_format == SWGB_FORMAT_R8G8B8A8_UNORM ? CF_RGBA8 : (st->color_format == SWGB_FORMAT_R16G16B16A16_SFLOAT ? CF_RGBA16F : CF_RGBA32F);
    D.color = (uint8_t *)st->color;
    D.colorPitch = st->color_pitch_bytes;
    D.depth = (uint8_t *)st->depth;
    D.depthPitch = st->depth_pitch_bytes;
    D.vec16 = ((uintptr_t)D.color % 16 == 0) && (D.colorPitch % 16 == 0) &&
              (!D.depthTest || (((uintptr_t)D.depth % 16 == 0) && (D.depthPitch % 16 == 0)));

    if(D.fs == SWGB_FS_TEX_X_VCOLOR)
    {
        const swgb_texture &t = st->texture;
        if(t.format == SWGB_FORMAT_R8G8B8A8_UNORM) D.texFloat = 0;
        else if(t.format == SWGB_FORMAT_R16G16B16A16_SFLOAT) D.texFloat = 1;
        else if(t.format == SWGB_FORMAT_R32G32B32A32_SFLOAT) D.texFloat = 2;
        else return set_error(SWGB_UNSUPPORTED_STATE, "texture format");
        if(t.level_count < 1 || t.level_count > SWGB_MAX_MIP_LEVELS) return set_error(SWGB_INVALID_ARG, "texture level_count");
        if(t.mag_filter != t.min_filter) return set_error(SWGB_UNSUPPORTED_STATE, "mixed min/mag filters");
        if(t.address_u > SWGB_ADDRESS_CLAMP_TO_EDGE || t.address_v > SWGB_ADDRESS_CLAMP_TO_EDGE) return set_error(SWGB_UNSUPPORTED_STATE, "address mode");
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
    }
    D.binX0 = D.sx0 & ~(BIN - 1);
    D.binY0 = D.sy0 & ~(BIN - 1);
    D.binsX = (D.sx1 - D.binX0 + BIN - 1) / BIN;
    D.binsY = (D.sy1 - D.binY0 + BIN - 1) / BIN;
    D.nchunks = (int)((a->count + CHUNK - 1) / CHUNK);
    D.nsuper = (D.nchunks + SUPER - 1) / SUPER;
    return SWGB_OK;
}

template<int CF, int MS>
constexpr size_t raster_smem() { return RASTER_WARPS * sizeof(RasterShared<CF, MS>); }

// Persistent raster grid of one kernel instantiation: SMs x resident blocks.
template<int CF, int MS>
swgb_status raster_grid(int device, bool setAttr, int &blocks)
{
    swgb_status s;
    if(setAttr && (s = cuda_check(cudaFuncSetAttribute(k_raster<CF, MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)raster_smem<CF, MS>()),
                                  "raster smem attribute")) != SWGB_OK)
        return s;
    int sms = 0, perSM = 0;
    if((s = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count")) != SWGB_OK) return s;
    if((s = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_raster<CF, MS>, RASTER_THREADS, raster_smem<CF, MS>()),
                       "raster occupancy")) != SWGB_OK)
        return s;
    blocks = (sms > 0 ? sms : 1) * (perSM > 0 ? perSM : 1);
    return SWGB_OK;
}

// Raster kernel index: colour format x (1 or 4 samples).
inline int raster_variant(const DrawParams &D) { return D.cf + (D.ms > 1 ? 3 : 0); }

swgb_status raster_grids(int device, bool setAttr, int blocks[6])
{
    swgb_status s;
    if((s = raster_grid<CF_RGBA8, 1>(device, setAttr, blocks[0])) != SWGB_OK) return s;
    if((s = raster_grid<CF_RGBA16F, 1>(device, setAttr, blocks[1])) != SWGB_OK) return s;
    if((s = raster_grid<CF_RGBA32F, 1>(device, setAttr, blocks[2])) != SWGB_OK) return s;
    if(!setAttr) return SWGB_OK;  // the allocation-free path runs single-sample draws only
    if((s = raster_grid<CF_RGBA8, 4>(device, setAttr, blocks[3])) != SWGB_OK) return s;
    if((s = raster_grid<CF_RGBA16F, 4>(device, setAttr, blocks[4])) != SWGB_OK) return s;
    return raster_grid<CF_RGBA32F, 4>(device, setAttr, blocks[5]);
}

void launch_raster(const DrawParams &D, uint32_t blocks, cudaStream_t st)
{
    switch(raster_variant(D))
    {
    case 0: k_raster<CF_RGBA8, 1><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA8, 1>(), st>>>(D); break;
    case 1: k_raster<CF_RGBA16F, 1><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA16F, 1>(), st>>>(D); break;
    case 2: k_raster<CF_RGBA32F, 1><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA32F, 1>(), st>>>(D); break;
    case 3: k_raster<CF_RGBA8, 4><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA8, 4>(), st>>>(D); break;
    case 4: k_raster<CF_RGBA16F, 4><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA16F, 4>(), st>>>(D); break;
    default: k_raster<CF_RGBA32F, 4><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA32F, 4>(), st>>>(D); break;
    }
}

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
void timed_launch(swgb_ctx *ctx, int kind, F &&launch)
{
    cudaEvent_t a = nullptr, b = nullptr;
    if(ctx->timing)
    {
        a = take_event(ctx);
        b = take_event(ctx);
        cudaEventRecord(a, ctx->stream);
    }
    launch();
    ctx->launches++;
    if(ctx->timing)
    {
        cudaEventRecord(b, ctx->stream);
        ctx->evPairs->push_back({kind, {a, b}});
    }
}

// Grows the context's scratch for draw D and points D at it.
swgb_status prepare_scratch(swgb_ctx *ctx, DrawParams &D)
{
    swgb_status s;
    if((s = ensure(ctx->ptv, ctx->ptvCap, (size_t)D.vertexCount * 4, "ptv")) != SWGB_OK) return s;
    const size_t triSlots = ((size_t)D.count + SETUP_THREADS - 1) / SETUP_THREADS * SETUP_THREADS;
    if((s = ensure(ctx->triBox, ctx->triBoxCap, triSlots, "triangle boxes")) != SWGB_OK) return s;
    if((s = ensure(ctx->triInfo, ctx->triInfoCap, triSlots, "triangle records")) != SWGB_OK) return s;
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
    if(!ctx->rasterAttr)
    {
        if((s = raster_grids(ctx->device, true, ctx->rasterBlocks)) != SWGB_OK) return s;
        ctx->rasterAttr = true;
    }
    return SWGB_OK;
}

swgb_status enqueue(swgb_ctx *ctx, DrawParams &D)
{
    if(D.count == 0) return SWGB_OK;  // Renderer.cpp:187
    swgb_status s;
    if((s = prepare_scratch(ctx, D)) != SWGB_OK) return s;
    const uint32_t nv = D.vertexCount;
    timed_launch(ctx, SWGB_KERNEL_VERTEX, [&] { k_vertex<<<(nv + 255) / 256, 256, 0, ctx->stream>>>(D, nv); });
    const uint32_t setupBlocks = (uint32_t)((D.count + SETUP_THREADS - 1) / SETUP_THREADS);
    timed_launch(ctx, SWGB_KERNEL_SETUP, [&] { k_setup<<<setupBlocks, SETUP_THREADS, 0, ctx->stream>>>(D); });
    if(D.binsX > 0 && D.binsY > 0)
    {
        uint32_t blocks = (uint32_t)((D.binsX * D.binsY + RASTER_WARPS - 1) / RASTER_WARPS);
        if(blocks > (uint32_t)ctx->rasterBlocks[raster_variant(D)]) blocks = (uint32_t)ctx->rasterBlocks[raster_variant(D)];
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
    cudaGraphExec_t graph[8] = {};  // raster variants 0-5, adjoint 1 / 4 samples
    uint64_t graphGen[8] = {};
    uint64_t gen = 1;
    cudaStream_t captureStream = nullptr;
    int vertexBlocks = 0, setupBlocks = 0;
    int rasterBlocks[6] = {};  // persistent grid per raster variant
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
        if(D.depthTest)
            plane_rects((uintptr_t)D.depth + (uintptr_t)q * D.depthSlice, origin, D.depthPitch, (int64_t)D.sx0 * 4,
                        (int64_t)D.sx1 * 4, D.sy0, D.sy1, out);
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
        const uintptr_t tb = st.texture.format == SWGB_FORMAT_R8G8B8A8_UNORM ? 4 : st.texture.format == SWGB_FORMAT_R16G16B16A16_SFLOAT ? 8 : 16;
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
    switch(variant)
    {
    case 0: k_raster_batch<CF_RGBA8, 1><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA8, 1>(), st>>>(P); break;
    case 1: k_raster_batch<CF_RGBA16F, 1><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA16F, 1>(), st>>>(P); break;
    case 2: k_raster_batch<CF_RGBA32F, 1><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA32F, 1>(), st>>>(P); break;
    case 3: k_raster_batch<CF_RGBA8, 4><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA8, 4>(), st>>>(P); break;
    case 4: k_raster_batch<CF_RGBA16F, 4><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA16F, 4>(), st>>>(P); break;
    default: k_raster_batch<CF_RGBA32F, 4><<<blocks, RASTER_THREADS, raster_smem<CF_RGBA32F, 4>(), st>>>(P); break;
    }
}

template<int CF, int MS>
swgb_status batch_attr(int sms, int &blocks)
{
    swgb_status s = cuda_check(cudaFuncSetAttribute(k_raster_batch<CF, MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)raster_smem<CF, MS>()),
                               "batch raster smem attribute");
    if(s != SWGB_OK) return s;
    int perSM = 0;
    if((s = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_raster_batch<CF, MS>, RASTER_THREADS, raster_smem<CF, MS>()),
                       "batch raster occupancy")) != SWGB_OK)
        return s;
    blocks = sms * (perSM > 0 ? perSM : 1);
    return SWGB_OK;
}

swgb_status batch_init(swgb_ctx *ctx)
{
    if(ctx->batch) return SWGB_OK;
    BatchState *B = new BatchState();
    swgb_status s;
    int sms = 1, perSM = 1;
    if((s = cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "SM count")) != SWGB_OK ||
       (s = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_setup_batch, SETUP_THREADS, 0), "setup occupancy")) != SWGB_OK ||
       (s = batch_attr<CF_RGBA8, 1>(sms, B->rasterBlocks[0])) != SWGB_OK || (s = batch_attr<CF_RGBA16F, 1>(sms, B->rasterBlocks[1])) != SWGB_OK ||
       (s = batch_attr<CF_RGBA32F, 1>(sms, B->rasterBlocks[2])) != SWGB_OK || (s = batch_attr<CF_RGBA8, 4>(sms, B->rasterBlocks[3])) != SWGB_OK ||
       (s = batch_attr<CF_RGBA16F, 4>(sms, B->rasterBlocks[4])) != SWGB_OK || (s = batch_attr<CF_RGBA32F, 4>(sms, B->rasterBlocks[5])) != SWGB_OK)
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
    cudaFree(B->ptv); cudaFree(B->ptv64); cudaFree(B->triBox); cudaFree(B->triInfo); cudaFree(B->chunk); cudaFree(B->super);
    cudaFree(B->spans); cudaFree(B->poly); cudaFree(B->queue); cudaFree(B->desc);
    if(B->stage) cudaFreeHost(B->stage);
    if(B->stageFree) cudaEventDestroy(B->stageFree);
    for(int v = 0; v < 8; v++)
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
        d.chunkBox = B.chunk + sOff / CHUNK;
        d.superBox = B.super + supOff;
        d.spans = B.spans;
        d.spanCount = ctx->spanCount;
        d.spanCapacity = ctx->spanRowsLimit ? std::min<uint64_t>(B.spansCap, ctx->spanRowsLimit) : B.spansCap;
        d.poly = B.poly;
        d.polyCount = ctx->polyCount;
        d.polyCapacity = (uint32_t)std::min<size_t>(B.polyCap / MAX_POLY, 0xFFFFFFFFu);
        d.counters = ctx->counters;
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
    // graph slot: raster variants 0-5, adjoint 6 (1 sample) and 7 (4 samples)
    const int variant = adj ? 6 + (draws[first].ms > 1 ? 1 : 0) : raster_variant(draws[first]);
    const uint32_t rblocks = (uint32_t)(adj ? ctx->adjBlocks[variant - 6] : B.rasterBlocks[variant]);
    auto third = [&](cudaStream_t st) {
        if(adj) launch_adjoint_batch(variant - 6, P, rblocks, st, ctx->adjScratch);
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
        if(args[i].count == 0) continue;  // Renderer.cpp:187
        DrawParams D;
        swgb_status s = bake(&states[i], &args[i], D);
        if(s != SWGB_OK) return s;
        draws.push_back(D);
        src.push_back(i);
    }
    if(draws.empty()) return SWGB_OK;
    swgb_status s;
    if((s = batch_init(ctx)) != SWGB_OK) return s;
    std::vector<std::pair<uint32_t, uint32_t>> segs;
    segment_batch(draws, src, states, args, segs);
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
    if(D.cf == CF_RGBA8) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint needs a float colour attachment");
    if(D.fs == SWGB_FS_TEX_X_VCOLOR && !D.texFloat) return set_error(SWGB_UNSUPPORTED_STATE, "adjoint needs a float texture");
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
    if((s = prepare_scratch(ctx, D)) != SWGB_OK) return s;
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
constexpr size_t NA_OFF_CHUNK = na_up(NA_OFF_INFO + (size_t)NA_SLOTS * sizeof(TriInfo));
constexpr size_t NA_OFF_SUPER = na_up(NA_OFF_CHUNK + (size_t)NA_CHUNKS * sizeof(short4));
constexpr size_t NA_OFF_SPANS = na_up(NA_OFF_SUPER + (size_t)NA_SUPER * sizeof(int4));
constexpr size_t NA_OFF_POLY = na_up(NA_OFF_SPANS + (size_t)NA_SPAN_ROWS * sizeof(uint32_t));
constexpr size_t NA_OFF_WORDS = na_up(NA_OFF_POLY + (size_t)NA_TRIS * MAX_POLY * sizeof(int2));
// words: counters[8] (u64), spanCount (u64), polyCount (u32), binQueue (u32), error (i32)
constexpr size_t NA_WORDS_BYTES = 8 * 8 + 8 + 4 + 4 + 4;
constexpr size_t NA_BYTES = na_up(NA_OFF_WORDS + NA_WORDS_BYTES);
static_assert(raster_smem<CF_RGBA32F, 1>() <= 48 * 1024 && raster_smem<CF_RGBA16F, 1>() <= 48 * 1024 && raster_smem<CF_RGBA8, 1>() <= 48 * 1024,
              "the allocation-free raster launch uses the default shared-memory limit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

struct NoAllocDevice {
    bool ready;
    unsigned char *base;  // device address of g_noalloc_scratch on this device
    int rasterBlocks[6];
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
        if((s = raster_grids(dev, false, d.rasterBlocks)) != SWGB_OK) return s;
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
    c->evFree = new std::vector<cudaEvent_t>();
    c->evPairs = new std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>>();
    if(stream)
        c->stream = (cudaStream_t)stream;
    else
    {
        if((s = cuda_check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream")) != SWGB_OK) { delete c; return s; }
        c->ownStream = true;
    }
    if(const char *lim = getenv("SWGB_SPAN_ROWS")) c->spanRowsLimit = strtoull(lim, nullptr, 10);
    if((s = cuda_check(cudaMalloc((void **)&c->polyCount, sizeof(uint32_t)), "polyCount")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->spanCount, sizeof(unsigned long long)), "spanCount")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->binQueue, sizeof(unsigned int)), "binQueue")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->counters, CTX_COUNTERS * sizeof(unsigned long long)), "counters")) != SWGB_OK ||
       (s = cuda_check(cudaMalloc((void **)&c->error, sizeof(int)), "error")) != SWGB_OK)
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
    cudaFree(c->triBox);
    cudaFree(c->triInfo);
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
    if(args->count == 0) return SWGB_OK;
    DrawParams D;
    swgb_status s = bake(st, args, D);
    if(s != SWGB_OK) return s;
    cudaSetDevice(ctx->device);
    return enqueue(ctx, D);
}

// The allocation-free variant of swgb_draw: the same validation, baking and
// kernels, with every scratch buffer carved out of g_noalloc_scratch.  It calls
// no cudaMalloc/cudaFree and no allocating library routine.
swgb_status swgb_draw_noalloc(const swgb_pipeline_state *st, const swgb_draw_args *args, void *stream)
{
    if(!st || !args) return set_error(SWGB_INVALID_ARG, "null argument");
    if(args->count == 0) return SWGB_OK;
    if(args->count > SWGB_NOALLOC_MAX_TRIANGLES)
        return set_error(SWGB_INVALID_ARG, "swgb_draw_noalloc: more than SWGB_NOALLOC_MAX_TRIANGLES (32768) triangles");
    DrawParams D;
    swgb_status s = bake(st, args, D);
    if(s != SWGB_OK) return s;
    if(D.ms > 1) return set_error(SWGB_UNSUPPORTED_STATE, "swgb_draw_noalloc: multisampled attachments need swgb_draw");
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
        if(blocks > (uint32_t)nd->rasterBlocks[D.cf]) blocks = (uint32_t)nd->rasterBlocks[D.cf];  // single-sample variants
        launch_raster(D, blocks, st0);
    }
    return cuda_check(cudaGetLastError(), "kernel launch");
}

swgb_status swgb_draw_batch(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n)
{
    if(!ctx || (!states && n) || (!args && n)) return set_error(SWGB_INVALID_ARG, "null argument");
    if(n == 0) return SWGB_OK;
    cudaSetDevice(ctx->device);
    return draw_batch(ctx, states, args, n);
}

swgb_status swgb_plan_batch(const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n, uint32_t *segment_first,
                            uint32_t *segment_count)
{
    if((n && (!states || !args)) || !segment_count) return set_error(SWGB_INVALID_ARG, "null argument");
    std::vector<DrawParams> draws;
    std::vector<uint32_t> src;
    for(uint32_t i = 0; i < n; i++)
    {
        if(args[i].count == 0) continue;
        DrawParams D;
        swgb_status s = bake(&states[i], &args[i], D);
        if(s != SWGB_OK) return s;
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
