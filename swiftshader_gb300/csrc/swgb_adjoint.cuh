// swgb_adjoint.cuh -- adjoint (backward) kernels of the draw path.
//
// Included by swgb_draw.cu inside its device namespace: it reuses the
// forward's vertex and setup stages (post-transform vertices, triangle boxes,
// span rows) and the raster stage's bin walk.  The reference has no backward
// pass; what is differentiated is stated in include/swgb.h (swgb_draw_adjoint).
//
// Per bin, one warp:
//   1. replays the draw's coverage and depth test in primitive order from the
//      clear depth: without blending it records the last writer of every
//      sample (shared memory); with blending it counts the passing fragments
//      of every pixel, then replays again per chunk of pixels whose fragments
//      fit the warp's region of the adjoint scratch, recording them grouped
//      by pixel in primitive order (no limit on fragments per pixel);
//   2. compares the replayed depth with the depth the draw left;
//   3. runs the adjoint of the blend over each sample's fragments and the
//      adjoint of shading for each (pixel, triangle): perspective-correct
//      barycentrics from the clip-space vertices, the fixed fragment shader
//      and the fp32 texture filter.  Texel gradients accumulate with float4
//      atomics, vertex-attribute and position gradients with fp32 atomics
//      (positions through the transpose of the draw's MVP).
#pragma once

constexpr int ADJ_WARPS = 2;  // bins (warps) per adjoint block
constexpr int ADJ_THREADS = 32 * ADJ_WARPS;
constexpr uint32_t ADJ_TRI_MASK = 0x0FFFFFFFu;  // entry = triangle | sample mask << 28
constexpr uint32_t ADJ_NO_WRITER = 0xFFFFFFFFu;
// Blended fragments a warp holds at once (its region of the adjoint
// scratch); a bin with more is processed in pixel chunks.
constexpr int ADJ_ENTRIES = 2048;
constexpr size_t ADJ_REGION_BYTES = (size_t)ADJ_ENTRIES * (4 + 4 + 4 + 4 + 16 + 16 + 16);

// Per-draw adjoint parameters, baked on the host from swgb_adjoint_args.
struct AdjParams {
    const uint8_t *gradColor;  // float RGBA per pixel and sample
    uint32_t gradPitch;
    uint64_t gradSlice;
    float clear[4];
    float clearDepth;
    int blendOver;  // premultiplied OVER (ONE, ONE_MINUS_SRC_ALPHA, ADD), else no blend
    float *gradTex[SWGB_MAX_MIP_LEVELS];   // float RGBA per texel, level pitch
    uint8_t *gradAttr[SWGB_MAX_ATTRIBS];   // binding gradient buffer + attribute offset
    uint32_t gradStride[SWGB_MAX_ATTRIBS];
    // clip-space ray of pixel centre (px, py): (rx0 + px rxs, ry0 + py rys, 1)
    double rx0, rxs, ry0, rys;
};

// A warp's region of the adjoint scratch: one blended fragment per entry,
// grouped by pixel in primitive order.
struct AdjRegion {
    uint32_t *tri;   // triangle | sample mask << 28
    uint32_t *pix;   // pixel index in the bin
    uint32_t *ltri;  // the same, in arrival order (the replay's log)
    uint32_t *lpix;
    float4 *sc;      // shaded colour
    float4 *ds;      // dL/d(shaded colour)
    float4 *before;  // colour of the sample before the fragment (one sample at a time)
    __device__ __forceinline__ explicit AdjRegion(uint8_t *base)
    {
        tri = (uint32_t *)base;
        pix = tri + ADJ_ENTRIES;
        ltri = pix + ADJ_ENTRIES;
        lpix = ltri + ADJ_ENTRIES;
        sc = (float4 *)(lpix + ADJ_ENTRIES);
        ds = sc + ADJ_ENTRIES;
        before = ds + ADJ_ENTRIES;
    }
};

template<int MS>
struct __align__(16) AdjShared {  // 16: the warps' copies sit back to back
    float depth[MS][BIN * BIN];  // replayed depth
    float4 planeA[BATCH][PLANES_STORED / 4];
    uint32_t span[BATCH][MS][BIN + 1];  // padded as in RasterShared
    int16_t qx0[BATCH][BIN / 2 + 2];
    uint16_t qpre[BATCH][BIN / 2 + 3];
    int8_t qr0[BATCH];
    int8_t nqr[BATCH];
    int8_t front[BATCH];  // facing (unused: the adjoint takes no stencil)
    int triList[2 * BATCH];
    uint32_t writer[MS][BIN * BIN];  // not blended: last fragment written per sample
    uint32_t off[BIN * BIN + 1];     // blended: first entry of each pixel (prefix of cnt)
    uint16_t cnt[BIN * BIN];         // blended: fragments per pixel
    uint16_t fill[BIN * BIN];        // blended: fragments recorded per pixel
    uint32_t logCount;               // blended: fragments appended to the region's log
    static constexpr int kSamples = MS;
    static constexpr int kBW = BIN, kBH = BIN;
    static constexpr bool kFull = false;  // the adjoint takes D32_SFLOAT depth, no bias, bounds or stencil
};

// A bin's pixels may be split between four warps (quarters of 8x8 pixels,
// sub = 0..3; sub = -1: the whole bin).  Pixel j of a part, in row order:
__device__ __forceinline__ bool in_sub(int idx, int sub)
{
    return sub < 0 || ((idx & (BIN - 1)) >> 3) + 2 * ((idx / BIN) >> 3) == sub;
}

__device__ __forceinline__ int sub_pixel(int j, int sub)
{
    if(sub < 0) return j;
    return ((sub >> 1) * 8 + (j >> 3)) * BIN + (sub & 1) * 8 + (j & 7);
}

__device__ __forceinline__ int sub_pixels(int sub) { return sub < 0 ? BIN * BIN : BIN * BIN / 4; }

// What a replay does with each passing (pixel, triangle, samples).
// REPLAY_LOG counts like REPLAY_COUNT and also appends every fragment to the
// region's log (arrival order keeps each pixel's primitive order) while it
// fits; REPLAY_RECORD is the fallback that records chunks of pixels.
enum { REPLAY_WRITERS = 0, REPLAY_COUNT = 1, REPLAY_RECORD = 2, REPLAY_LOG = 3 };

// Replay of one batch of nb <= 32 triangles: coverage per sample (the
// forward's spans), depth test against the replayed depth in primitive
// order.  Lanes are quad slots in primitive order; lanes on the same quad
// resolve lowest lane (earliest triangle) first, so per-pixel state needs no
// atomics.  REPLAY_RECORD stores the fragments of pixels [p0, p1) at
// S.off[idx] - S.off[p0] + (running count) of the region.
template<int MS>
__device__ __noinline__ void adjoint_replay(const DrawParams &D, AdjShared<MS> &S, AdjRegion R, int MODE, int nb, int bx0,
                                            int by0, int p0, int p1, int sub, unsigned long long &nOverflow)
{
    const int lane = threadIdx.x & 31;
    int cnt = 0;
    if(lane < nb) cnt = setup_batch_triangle(D, S, lane, (uint32_t)S.triList[lane], bx0, by0);
    __syncwarp();
    const bool earlyZ = D.depthTest && (D.compareOp == SWGB_COMPARE_LESS || D.compareOp == SWGB_COMPARE_LESS_OR_EQUAL ||
                                        D.compareOp == SWGB_COMPARE_GREATER || D.compareOp == SWGB_COMPARE_GREATER_OR_EQUAL);
    const int incl = warp_incl_scan(cnt, lane);
    const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    const uint32_t base = MODE == REPLAY_RECORD ? S.off[p0] : 0u;
    for(int s0 = 0; s0 < total; s0 += 32)
    {
        const int slot = s0 + lane;
        int src;
        {
            int lo = 0, hi = 31;
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
        int cMask = 0, qx = 0, qrow = 0;
        const int qti = src;
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
                int m = 0;
                if(qx >= l0 && qx < r0) m |= 1;
                if(qx + 1 >= l0 && qx + 1 < r0) m |= 2;
                if(qx >= l1 && qx < r1) m |= 4;
                if(qx + 1 >= l1 && qx + 1 < r1) m |= 8;
                cMask |= m << (4 * q);
            }
            if(cMask && earlyZ)
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
                cMask = keep;
            }
        }
        const int key = cMask ? qrow * BIN + (qx - bx0) : -1 - lane;
        unsigned pend = __ballot_sync(0xFFFFFFFFu, cMask != 0);
        while(pend)
        {
            const bool mine = (pend >> lane) & 1;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, mine ? key : -1 - lane);
            if(mine && (__ffs(peers) - 1) == lane)
            {
                const uint32_t tri = (uint32_t)S.triList[qti];
                const int y = by0 + 2 * qrow;
#pragma unroll
                for(int i = 0; i < 4; i++)
                {
                    const int idx = (2 * qrow + (i >> 1)) * BIN + (qx - bx0) + (i & 1);
                    uint32_t m = 0;
#pragma unroll
                    for(int q = 0; q < MS; q++)
                    {
                        if(!(cMask >> (4 * q + i) & 1)) continue;
                        if(D.depthTest)
                        {
                            const float z = sample_depth<MS>(D, S, qti, qx, y, i, q);
                            if(!depth_pass(D.compareOp, S.depth[q][idx], z)) continue;
                            if(D.depthWrite) S.depth[q][idx] = z;
                        }
                        m |= 1u << q;
                    }
                    if(!m) continue;
                    if(MODE == REPLAY_WRITERS)
                    {
#pragma unroll
                        for(int q = 0; q < MS; q++)
                            if(m >> q & 1) S.writer[q][idx] = tri;
                    }
                    else if(!in_sub(idx, sub))
                        continue;
                    else if(MODE == REPLAY_COUNT || MODE == REPLAY_LOG)
                    {
                        S.cnt[idx] = (uint16_t)min((int)S.cnt[idx] + 1, 0xFFFF);
                        if(MODE == REPLAY_LOG)
                        {
                            const uint32_t pos = atomicAdd(&S.logCount, 1u);
                            if(pos < (uint32_t)ADJ_ENTRIES)
                            {
                                R.ltri[pos] = tri | (m << 28);
                                R.lpix[pos] = (uint32_t)idx;
                            }
                        }
                    }
                    else if(idx >= p0 && idx < p1)
                    {
                        const uint32_t pos = S.off[idx] - base + S.fill[idx];
                        S.fill[idx]++;
                        if(pos < (uint32_t)ADJ_ENTRIES)
                        {
                            R.tri[pos] = tri | (m << 28);
                            R.pix[pos] = (uint32_t)idx;
                        }
                        else
                            nOverflow++;
                    }
                }
                pend &= ~(1u << lane);
            }
            __syncwarp();
            pend = __ballot_sync(0xFFFFFFFFu, mine && ((pend >> lane) & 1));
        }
    }
    __syncwarp();
}

// ---- shading model ---------------------------------------------------------
//
// The geometric part of the model -- homogeneous barycentrics, interpolated
// varyings, texture addresses and the position gradient -- runs in fp64:
// the position gradient sums per-pixel terms that cancel, and the derivative
// of bilinear filtering jumps at texel centres, so fp32 coordinates (1e-5
// texel error at 128 texels) move it by more than the 1e-4 the gradients
// are held to.  Texel values, colours and atomics stay fp32.

// A triangle's post-transform vertices: slots, clip (x, y, w) and varyings.
struct AdjTri {
    uint32_t slot[3];
    double3 q[3];
    double2 proj[3];  // (x / w, y / w); 0 when w = 0
    float var[3][MAXV];
};

__device__ __noinline__ void adj_load_tri(const DrawParams &D, uint32_t t, AdjTri &T)
{
    tri_slots(D, t, T.slot[0], T.slot[1], T.slot[2]);
#pragma unroll
    for(int i = 0; i < 3; i++)
    {
        // clip (x, y, w) = MVP p and its projection, fp64, from the vertex
        // stage: the forward's fp32 clip coordinates would move the position
        // gradient by ~1e-4
        const double *c = D.ptv64 + (size_t)T.slot[i] * 6;
        T.q[i] = make_double3(c[0], c[1], c[2]);
        T.proj[i] = make_double2(c[3], c[4]);
        const float4 a = D.ptv[(size_t)T.slot[i] * 4 + 2], b = D.ptv[(size_t)T.slot[i] * 4 + 3];
        T.var[i][0] = a.y; T.var[i][1] = a.z; T.var[i][2] = a.w;
        T.var[i][3] = b.x; T.var[i][4] = b.y; T.var[i][5] = b.z; T.var[i][6] = b.w;
    }
}

__device__ __forceinline__ double3 cross3(double3 a, double3 b)
{
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ double3 sub3(double3 a, double3 b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }

// Clip-space ray of the centre of pixel (px, py): the sample point of pixel
// px is X = 256 px in the fixed-point frame X = X0xF + x_ndc * WxF, so
// x_ndc = px * 256 / WxF - X0xF / WxF (the two constants baked in AdjParams).
__device__ __forceinline__ double3 pixel_ray(const AdjParams &A, int px, int py)
{
    return make_double3(fma((double)px, A.rxs, A.rx0), fma((double)py, A.rys, A.ry0), 1.0);
}

// address_float in fp64 with its slope: x0, x1, the filter fraction f and
// d(coordinate * dim)/du.
__device__ __forceinline__ void address_fp64(const DrawParams &D, double coord, uint32_t mode, int dim, int32_t &x0, int32_t &x1,
                                             float &f, float &slope)
{
    const double one = (double)__int_as_float(0x3F7FFFFF);
    double c;
    if(mode == SWGB_ADDRESS_CLAMP_TO_EDGE)
    {
        c = fmin(fmax(coord, 0.0), one);
        slope = (coord > 0.0 && coord < 1.0) ? 1.0f : 0.0f;
    }
    else if(mode == SWGB_ADDRESS_MIRRORED_REPEAT)
    {
        const double h = coord * 0.5, d = h - rint(h);
        c = fmin(2.0 * fabs(d), one);
        slope = d > 0.0 ? 1.0f : (d < 0.0 ? -1.0f : 0.0f);
    }
    else
    {
        c = fmin(coord - floor(coord), one);
        slope = 1.0f;
    }
    slope *= (float)dim;
    c *= dim;
    if(!D.texLinear)
    {
        x0 = x1 = (int32_t)floor(c);
        f = 0.0f;
        return;
    }
    c -= 0.5;
    const double fl = floor(c);
    x0 = (int32_t)fl;
    f = (float)(c - fl);
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

__device__ __forceinline__ float4 f4_lerp(float4 a, float4 b, float t)
{
    return make_float4(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z), a.w + t * (b.w - a.w));
}

__device__ __forceinline__ float4 f4_axpy(float a, float4 x, float4 y)
{
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}

__device__ __forceinline__ void grad_texel(float *g, int32_t index, float w, const float gt[4])
{
    if(w == 0.0f) return;
    atomicAdd(reinterpret_cast<float4 *>(g) + (uint32_t)index, make_float4(w * gt[0], w * gt[1], w * gt[2], w * gt[3]));
}

// The filter at (u, v) with the level of detail fixed: the filtered texel,
// its derivatives by u and v, and (when gt != nullptr) the texel gradients
// gt * filter weight accumulated into the level gradients.
__device__ __noinline__ void adj_filter(const DrawParams &D, const AdjParams &A, double u, double v, float lod, const float *gt,
                                        float4 &tex, float4 &dtdu, float4 &dtdv)
{
    tex = dtdu = dtdv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int levels = D.mipLinear ? 2 : 1;
    const float fr = lod - floorf(lod);
    for(int second = 0; second < levels; second++)
    {
        const float wl = D.mipLinear ? (second ? fr : 1.0f - fr) : 1.0f;
        int ilod = D.mipLinear ? trunc_int(lod) : round_int(lod);
        int li = ilod + second;
        li = li < 0 ? 0 : (li > D.levelCount - 1 ? D.levelCount - 1 : li);
        const TexLevel &lv = D.lv[li];
        float *g = gt ? A.gradTex[li] : nullptr;
        int32_t x0, x1, y0, y1;
        float fu, fv, su, sv;
        address_fp64(D, u, D.addrU, (int)lv.w, x0, x1, fu, su);
        address_fp64(D, v, D.addrV, (int)lv.h, y0, y1, fv, sv);
        const int32_t pitch = (int32_t)lv.pitch;
        y0 *= pitch;
        if(!D.texLinear)
        {
            tex = f4_axpy(wl, texel_float(D, lv, x0 + y0), tex);
            if(g) grad_texel(g, x0 + y0, wl, gt);
            continue;
        }
        y1 *= pitch;
        const float4 c00 = texel_float(D, lv, x0 + y0), c10 = texel_float(D, lv, x1 + y0);
        const float4 c01 = texel_float(D, lv, x0 + y1), c11 = texel_float(D, lv, x1 + y1);
        const float4 a0 = f4_lerp(c00, c10, fu), a1 = f4_lerp(c01, c11, fu);
        tex = f4_axpy(wl, f4_lerp(a0, a1, fv), tex);
        const float4 du = f4_lerp(make_float4(c10.x - c00.x, c10.y - c00.y, c10.z - c00.z, c10.w - c00.w),
                                  make_float4(c11.x - c01.x, c11.y - c01.y, c11.z - c01.z, c11.w - c01.w), fv);
        dtdu = f4_axpy(wl * su, du, dtdu);
        dtdv = f4_axpy(wl * sv, make_float4(a1.x - a0.x, a1.y - a0.y, a1.z - a0.z, a1.w - a0.w), dtdv);
        if(g)
        {
            grad_texel(g, x0 + y0, wl * (1.0f - fu) * (1.0f - fv), gt);
            grad_texel(g, x1 + y0, wl * fu * (1.0f - fv), gt);
            grad_texel(g, x0 + y1, wl * (1.0f - fu) * fv, gt);
            grad_texel(g, x1 + y1, wl * fu * fv, gt);
        }
    }
}

// Interpolation state of triangle T at pixel (px, py): the homogeneous
// barycentrics b_i = u_i / U, u_i = r . (q_j x q_k), written with
// K_i = q_j x (q_k - q_j) and r replaced by d_j = r - q_j / w_j (same
// determinant), the pixel's offset from vertex j's projection.
struct AdjInterp {
    double3 r, d[3], K[3];
    double b[3], invU;
    double val[MAXV];  // interpolated varyings
    float lod;
    bool ok;
};

__device__ __noinline__ void adj_interp(const DrawParams &D, const AdjParams &A, const AdjTri &T, int px, int py, AdjInterp &I)
{
    I.K[0] = cross3(T.q[1], sub3(T.q[2], T.q[1]));
    I.K[1] = cross3(T.q[2], sub3(T.q[0], T.q[2]));
    I.K[2] = cross3(T.q[0], sub3(T.q[1], T.q[0]));
    I.r = pixel_ray(A, px, py);
#pragma unroll
    for(int j = 0; j < 3; j++) I.d[j] = make_double3(I.r.x - T.proj[j].x, I.r.y - T.proj[j].y, T.q[j].z != 0.0 ? 0.0 : 1.0);
    double uu[3];
#pragma unroll
    for(int i = 0; i < 3; i++) uu[i] = dot3(I.d[(i + 1) % 3], I.K[i]);
    const double U = uu[0] + uu[1] + uu[2];
    I.ok = U != 0.0 && isfinite(U);
    I.invU = I.ok ? 1.0 / U : 0.0;
#pragma unroll
    for(int i = 0; i < 3; i++) I.b[i] = uu[i] * I.invU;
#pragma unroll
    for(int k = 0; k < MAXV; k++) I.val[k] = I.b[0] * T.var[0][k] + I.b[1] * T.var[1][k] + I.b[2] * T.var[2][k];
    I.lod = D.minLod;
    if(D.fs == SWGB_FS_TEX_X_VCOLOR && I.ok && D.minLod != D.maxLod)
    {
        // level of detail from lanes 0, 1, 2 of the pixel's quad (it is held
        // constant; only its value is used): the lanes' texture coordinates
        // under the model in fp64, rounded to fp32, then the forward's fp32
        // LOD arithmetic.  In fp32 throughout, the coordinate differences
        // of a 2048^2 texture carried enough rounding to move the trilinear
        // weights by ~1e-4.
        const int qx = px & ~1, qy = py & ~1;
        float lu[4], lv[4];
#pragma unroll
        for(int j = 0; j < 3; j++)
        {
            // w_i = d_k . K_i with d_k the lane's offset from vertex k's projection
            const double3 rd = pixel_ray(A, qx + (j & 1), qy + (j >> 1));
            double w[3];
#pragma unroll
            for(int i = 0; i < 3; i++)
            {
                const int k = (i + 1) % 3;
                const double dx = rd.x - T.proj[k].x, dy = rd.y - T.proj[k].y;
                w[i] = dx * I.K[i].x + dy * I.K[i].y + (T.q[k].z != 0.0 ? 0.0 : I.K[i].z);
            }
            const double ws = w[0] + w[1] + w[2];
            lu[j] = (float)((w[0] * (double)T.var[0][4] + w[1] * (double)T.var[1][4] + w[2] * (double)T.var[2][4]) / ws);
            lv[j] = (float)((w[0] * (double)T.var[0][5] + w[1] * (double)T.var[1][5] + w[2] * (double)T.var[2][5]) / ws);
        }
        lu[3] = lu[0];
        lv[3] = lv[0];
        I.lod = implicit_lod(D, lu, lv);
    }
}

// Forward colour of triangle T at pixel (px, py) under the model.
__device__ __noinline__ float4 adj_shade(const DrawParams &D, const AdjParams &A, const AdjTri &T, int px, int py)
{
    AdjInterp I;
    adj_interp(D, A, T, px, py, I);
    float4 c = make_float4((float)I.val[0], (float)I.val[1], (float)I.val[2], (float)I.val[3]);
    if(D.fs == SWGB_FS_TEX_X_VCOLOR && I.ok)
    {
        float4 tex, du, dv;
        adj_filter(D, A, I.val[4], I.val[5], I.lod, nullptr, tex, du, dv);
        c = make_float4(tex.x * c.x, tex.y * c.y, tex.z * c.z, tex.w * c.w);
    }
    return c;
}

__device__ __forceinline__ void grad_attr(const AdjParams &A, int a, uint32_t index, int c, float g)
{
    if(A.gradAttr[a] && g != 0.0f) atomicAdd((float *)(A.gradAttr[a] + (size_t)index * A.gradStride[a]) + c, g);
}

// Adjoint of shading triangle T at pixel (px, py) given dL/d(shaded colour)
// gS: texel gradients, then dL/d(varyings) and dL/d(barycentrics), then
// dL/d(clip x, y, w) of the three vertices through b_i = u_i / U, and
// dL/d(position) = MVP^T dL/d(clip).
__device__ __noinline__ void adj_shade_grad(const DrawParams &D, const AdjParams &A, const AdjTri &T, int px, int py, float4 gS4)
{
    AdjInterp I;
    adj_interp(D, A, T, px, py, I);
    if(!I.ok) return;
    const float gS[4] = {gS4.x, gS4.y, gS4.z, gS4.w};
    // dL/d(varying k) of the pixel; varyings 0-3 colour, 4-5 texture coordinates
    float gvar[MAXV] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if(D.fs == SWGB_FS_TEX_X_VCOLOR)
    {
        const float gt[4] = {gS[0] * (float)I.val[0], gS[1] * (float)I.val[1], gS[2] * (float)I.val[2], gS[3] * (float)I.val[3]};
        float4 tex, du, dv;
        adj_filter(D, A, I.val[4], I.val[5], I.lod, gt, tex, du, dv);
        gvar[0] = gS[0] * tex.x; gvar[1] = gS[1] * tex.y; gvar[2] = gS[2] * tex.z; gvar[3] = gS[3] * tex.w;
        gvar[4] = gt[0] * du.x + gt[1] * du.y + gt[2] * du.z + gt[3] * du.w;
        gvar[5] = gt[0] * dv.x + gt[1] * dv.y + gt[2] * dv.z + gt[3] * dv.w;
    }
    else
    {
#pragma unroll
        for(int k = 0; k < 4; k++) gvar[k] = gS[k];
    }
    // dL/du_i = (dL/db_i - sum_m b_m dL/db_m) / U = sum_k gvar_k (var_i[k] - val[k]) / U
    double gU[3];
#pragma unroll
    for(int i = 0; i < 3; i++)
    {
        double s = 0.0;
#pragma unroll
        for(int k = 0; k < 6; k++) s += (double)gvar[k] * ((double)T.var[i][k] - I.val[k]);
        gU[i] = s * I.invU;
    }
    // d u_i / d q_j = q_k x r, d u_i / d q_k = r x q_j for (i, j, k) cyclic;
    // r x q_k = d_k x q_k
    double3 gq[3];
    {
        const double3 rq0 = cross3(I.d[0], T.q[0]), rq1 = cross3(I.d[1], T.q[1]), rq2 = cross3(I.d[2], T.q[2]);
        gq[0] = make_double3(gU[1] * rq2.x - gU[2] * rq1.x, gU[1] * rq2.y - gU[2] * rq1.y, gU[1] * rq2.z - gU[2] * rq1.z);
        gq[1] = make_double3(gU[2] * rq0.x - gU[0] * rq2.x, gU[2] * rq0.y - gU[0] * rq2.y, gU[2] * rq0.z - gU[0] * rq2.z);
        gq[2] = make_double3(gU[0] * rq1.x - gU[1] * rq0.x, gU[0] * rq1.y - gU[1] * rq0.y, gU[0] * rq1.z - gU[1] * rq0.z);
    }
#pragma unroll 1
    for(int i = 0; i < 3; i++)
    {
        const uint32_t index = (D.indexType == SWGB_INDEX_TYPE_NONE ? D.firstVertex + T.slot[i] : T.slot[i]) + (uint32_t)D.baseVertex;
        // position: clip = MVP p (column-major), so dL/dp_c = sum_r MVP[r][c] dL/dclip_r; z gets none
        const float gx = (float)gq[i].x, gy = (float)gq[i].y, gw = (float)gq[i].z;
        for(int c = 0; c < (int)D.vcomp[0]; c++)
            grad_attr(A, 0, index, c, D.mvp[4 * c] * gx + D.mvp[4 * c + 1] * gy + D.mvp[4 * c + 3] * gw);
        int k = 0;
        for(int a = 1; a < D.nattr; a++)
            for(int c = 0; c < (int)D.vcomp[a] && k < MAXV; c++, k++)
                grad_attr(A, a, index, c, (float)I.b[i] * gvar[k]);
    }
}

__device__ __forceinline__ float4 grad_color_at(const AdjParams &A, int q, int px, int py)
{
    return *(const float4 *)(A.gradColor + (size_t)q * A.gradSlice + (size_t)py * A.gradPitch + (size_t)px * 16);
}

// Not blended: each sample's colour is its last writer's shaded colour, so a
// writer of several samples takes the sum of their gradients.  The (pixel,
// writer, samples) entries are gathered into the region first, then shaded
// with lanes over entries (a pixel has up to MS of them).
template<int MS>
__device__ void adjoint_pixels_writers(const DrawParams &D, const AdjParams &A, AdjShared<MS> &S, AdjRegion R, int bx0, int by0,
                                       int sub, unsigned long long &nFrag)
{
    const int lane = threadIdx.x & 31;
    int nE = 0;  // warp-uniform
    for(int j0 = 0; j0 < sub_pixels(sub); j0 += 32)
    {
        const int idx = sub_pixel(j0 + lane, sub);
        uint32_t ent[MS];
        int ne = 0;
#pragma unroll
        for(int q = 0; q < MS; q++)
        {
            const uint32_t w = S.writer[q][idx];
            bool first = w != ADJ_NO_WRITER;
#pragma unroll
            for(int p = 0; p < q; p++) first = first && S.writer[p][idx] != w;
            if(!first) continue;
            uint32_t m = 0;
#pragma unroll
            for(int p = q; p < MS; p++)
                if(S.writer[p][idx] == w) m |= 1u << p;
            ent[ne++] = w | (m << 28);
        }
        const int incl = warp_incl_scan(ne, lane);
        const int base = nE + incl - ne;
#pragma unroll
        for(int k = 0; k < MS; k++)
            if(k < ne)
            {
                R.tri[base + k] = ent[k];
                R.pix[base + k] = (uint32_t)idx;
            }
        nE += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    __syncwarp();
    for(int e = lane; e < nE; e += 32)
    {
        const uint32_t v = R.tri[e];
        const int idx = (int)R.pix[e];
        const int px = bx0 + (idx % BIN), py = by0 + idx / BIN;
        float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for(int q = 0; q < MS; q++)
            if(v >> (28 + q) & 1)
            {
                const float4 G = grad_color_at(A, q, px, py);
                g = make_float4(g.x + G.x, g.y + G.y, g.z + G.z, g.w + G.w);
            }
        AdjTri T;
        adj_load_tri(D, v & ADJ_TRI_MASK, T);
        adj_shade_grad(D, A, T, px, py, g);
        nFrag++;
    }
    __syncwarp();
}

// Blended, pixels [p0, p1) of the bin whose fragments are in the region:
// shade every fragment (lanes over fragments), run the adjoint of
// C_e = S_e + (1 - S_e.a) C_{e-1} per sample (lanes over pixels), then the
// shading adjoint of every fragment (lanes over fragments).
template<int MS>
__device__ void adjoint_pixels_blended(const DrawParams &D, const AdjParams &A, AdjShared<MS> &S, AdjRegion R, int bx0, int by0,
                                       int p0, int p1, unsigned long long &nFrag)
{
    const int lane = threadIdx.x & 31;
    const uint32_t base = S.off[p0];
    const int nE = (int)min(S.off[p1] - base, (uint32_t)ADJ_ENTRIES);
    for(int e = lane; e < nE; e += 32)
    {
        const int idx = (int)R.pix[e];
        AdjTri T;
        adj_load_tri(D, R.tri[e] & ADJ_TRI_MASK, T);
        R.sc[e] = adj_shade(D, A, T, bx0 + (idx % BIN), by0 + idx / BIN);
        R.ds[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncwarp();
    for(int idx = p0 + lane; idx < p1; idx += 32)
    {
        const int e0 = (int)(S.off[idx] - base);
        const int e1 = min((int)(S.off[idx + 1] - base), ADJ_ENTRIES);
        if(e0 >= e1) continue;
        const int px = bx0 + (idx % BIN), py = by0 + idx / BIN;
#pragma unroll 1
        for(int q = 0; q < MS; q++)
        {
            float4 C = make_float4(A.clear[0], A.clear[1], A.clear[2], A.clear[3]);
            for(int e = e0; e < e1; e++)
                if(R.tri[e] >> (28 + q) & 1)
                {
                    R.before[e] = C;
                    const float4 Sc = R.sc[e];
                    const float t = 1.0f - Sc.w;
                    C = make_float4(Sc.x + t * C.x, Sc.y + t * C.y, Sc.z + t * C.z, Sc.w + t * C.w);
                }
            float4 g = grad_color_at(A, q, px, py);
            for(int e = e1 - 1; e >= e0; e--)
                if(R.tri[e] >> (28 + q) & 1)
                {
                    const float4 b = R.before[e], Sc = R.sc[e];
                    const float dot = g.x * b.x + g.y * b.y + g.z * b.z + g.w * b.w;
                    float4 d = R.ds[e];
                    R.ds[e] = make_float4(d.x + g.x, d.y + g.y, d.z + g.z, d.w + g.w - dot);
                    const float t = 1.0f - Sc.w;
                    g = make_float4(t * g.x, t * g.y, t * g.z, t * g.w);
                }
        }
    }
    __syncwarp();
    for(int e = lane; e < nE; e += 32)
    {
        const int idx = (int)R.pix[e];
        AdjTri T;
        adj_load_tri(D, R.tri[e] & ADJ_TRI_MASK, T);
        adj_shade_grad(D, A, T, bx0 + (idx % BIN), by0 + idx / BIN, R.ds[e]);
        nFrag++;
    }
    __syncwarp();
}

template<int MS>
__device__ __forceinline__ void adj_reset(const AdjParams &A, AdjShared<MS> &S)
{
    const int lane = threadIdx.x & 31;
    for(int i = lane; i < BIN * BIN; i += 32)
    {
#pragma unroll
        for(int q = 0; q < MS; q++) S.depth[q][i] = A.clearDepth;
        S.fill[i] = 0;
    }
    __syncwarp();
}

// Counters of the adjoint kernels: fragments, depth mismatches, overflows.
struct AdjCount {
    unsigned long long frag = 0, mismatch = 0, overflow = 0;
};

// One bin: replay(s) from the clear state, the replayed depth checked against
// the saved depth, then the pixels.
template<int MS>
__device__ __forceinline__ void adjoint_bin(const DrawParams &D, const AdjParams &A, AdjShared<MS> &S, AdjRegion R, int bin,
                                            int sub, AdjCount &n)
{
    const int lane = threadIdx.x & 31;
    const int bx0 = D.binX0 + (bin % D.binsX) * BIN;
    const int by0 = D.binY0 + (bin / D.binsX) * BIN;
    const bool over = A.blendOver != 0;
    adj_reset(A, S);
    for(int i = lane; i < BIN * BIN; i += 32)
    {
#pragma unroll
        for(int q = 0; q < MS; q++) S.writer[q][i] = ADJ_NO_WRITER;
        S.cnt[i] = 0;
    }
    if(lane == 0) S.logCount = 0;
    __syncwarp();
    if(over)
        walk_bin(D, S, bx0, by0, [&](int nb) { adjoint_replay<MS>(D, S, R, REPLAY_LOG, nb, bx0, by0, 0, 0, sub, n.overflow); });
    else
        walk_bin(D, S, bx0, by0, [&](int nb) { adjoint_replay<MS>(D, S, R, REPLAY_WRITERS, nb, bx0, by0, 0, 0, sub, n.overflow); });
    // the replay must end where the draw ended
    for(int j = lane; j < sub_pixels(sub); j += 32)
    {
        const int idx = sub_pixel(j, sub);
        const int px = bx0 + (idx % BIN), py = by0 + idx / BIN;
        if(!D.depthTest || !D.depthWrite || px < D.sx0 || px >= D.sx1 || py < D.sy0 || py >= D.sy1) continue;
#pragma unroll
        for(int q = 0; q < MS; q++)
        {
            const float saved = *(const float *)(D.depth + (size_t)q * D.depthSlice + (size_t)py * D.depthPitch + (size_t)px * 4);
            if(__float_as_uint(saved) != __float_as_uint(S.depth[q][idx])) n.mismatch++;
        }
    }
    if(!over)
    {
        adjoint_pixels_writers<MS>(D, A, S, R, bx0, by0, sub, n.frag);
        return;
    }
    // fragments per pixel -> first entry per pixel (8 pixels per lane)
    {
        uint32_t loc[8], sum = 0;
#pragma unroll
        for(int k = 0; k < 8; k++)
        {
            loc[k] = sum;
            sum += S.cnt[lane * 8 + k];
        }
        uint32_t incl = sum;
#pragma unroll
        for(int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if(lane >= o) incl += v;
        }
        const uint32_t excl = incl - sum;
#pragma unroll
        for(int k = 0; k < 8; k++) S.off[lane * 8 + k] = excl + loc[k];
        if(lane == 31) S.off[BIN * BIN] = incl;
    }
    __syncwarp();
    if(S.off[BIN * BIN] == 0) return;
    if(S.logCount <= (uint32_t)ADJ_ENTRIES)
    {
        // the log holds every fragment: stable scatter into pixel order (lanes
        // on one pixel take consecutive slots in lane order)
        for(int e0 = 0; e0 < (int)S.logCount; e0 += 32)
        {
            const int e = e0 + lane;
            const bool valid = e < (int)S.logCount;
            const uint32_t pix = valid ? R.lpix[e] : 0x10000u + lane;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, pix);
            if(valid)
            {
                const uint32_t pos = S.off[pix] + S.fill[pix] + __popc(peers & ((1u << lane) - 1u));
                R.tri[pos] = R.ltri[e];
                R.pix[pos] = pix;
            }
            __syncwarp();
            if(valid && (peers >> lane) == 1u) S.fill[pix] += (uint16_t)__popc(peers);
            __syncwarp();
        }
        adjoint_pixels_blended<MS>(D, A, S, R, bx0, by0, 0, BIN * BIN, n.frag);
        return;
    }
    // more fragments than the region holds: pixel chunks that fit it, one
    // replay each
    int p0 = 0;
    while(p0 < BIN * BIN)
    {
        int p1 = p0 + 1;
        while(p1 < BIN * BIN && S.off[p1 + 1] - S.off[p0] <= (uint32_t)ADJ_ENTRIES) p1++;
        if(S.off[p1] > S.off[p0])
        {
            adj_reset(A, S);
            walk_bin(D, S, bx0, by0, [&](int nb) { adjoint_replay<MS>(D, S, R, REPLAY_RECORD, nb, bx0, by0, p0, p1, sub, n.overflow); });
            adjoint_pixels_blended<MS>(D, A, S, R, bx0, by0, p0, p1, n.frag);
        }
        p0 = p1;
    }
}

__device__ __forceinline__ void flush_adjoint_counters(unsigned long long *counters, const AdjCount &n)
{
    const int lane = threadIdx.x & 31;
    const unsigned long long v3[3] = {n.frag, n.mismatch, n.overflow};
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
        unsigned long long v = v3[k];
#pragma unroll
        for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if(lane == 0 && v) atomicAdd(&counters[CNT_ADJ_FRAGMENTS + k], v);
    }
}

__device__ __forceinline__ uint8_t *adj_region_base(uint8_t *scratch)
{
    return scratch + (size_t)(blockIdx.x * ADJ_WARPS + (threadIdx.x >> 5)) * ADJ_REGION_BYTES;
}

// Work item k of a draw: bin k / split, part k % split (split 1: whole bins,
// split 4: quarters, for frames with fewer bins than resident warps).
template<int MS>
__global__ void __launch_bounds__(ADJ_THREADS) k_adjoint(const __grid_constant__ DrawParams D, const __grid_constant__ AdjParams A,
                                                         uint8_t *scratch, int split)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    AdjShared<MS> &S = reinterpret_cast<AdjShared<MS> *>(smem_raw)[threadIdx.x >> 5];
    const AdjRegion R(adj_region_base(scratch));
    const int lane = threadIdx.x & 31;
    const int items = D.binsX * D.binsY * split;
    AdjCount n;
    for(;;)
    {
        int item = 0;
        if(lane == 0) item = (int)atomicAdd(D.binQueue, 1u);
        item = __shfl_sync(0xFFFFFFFFu, item, 0);
        if(item >= items) break;
        adjoint_bin<MS>(D, A, S, R, item / split, split > 1 ? item % split : -1, n);
    }
    flush_adjoint_counters(D.counters, n);
}

// Adjoints of a batch of draws: bins of all draws in one queue; per-draw
// AdjParams follow the draw records in the batch descriptor.
template<int MS>
__global__ void __launch_bounds__(ADJ_THREADS) k_adjoint_batch(const __grid_constant__ BatchPtrs B, uint8_t *scratch)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    AdjShared<MS> &S = reinterpret_cast<AdjShared<MS> *>(smem_raw)[threadIdx.x >> 5];
    const AdjRegion R(adj_region_base(scratch));
    const int lane = threadIdx.x & 31;
    const BatchView V(B.hdr);
    const AdjParams *adj = (const AdjParams *)((const uint8_t *)B.hdr + V.h.offAdj);
    const uint32_t split = V.h.split ? V.h.split : 1;
    AdjCount n;
    for(;;)
    {
        uint32_t item = 0;
        if(lane == 0) item = atomicAdd(B.binQueue, 1u);
        item = __shfl_sync(0xFFFFFFFFu, item, 0);
        if(item >= V.h.bins * split) break;
        const uint32_t bin = item / split;
        const uint32_t d = find_draw(V.bStart, V.h.n, bin);
        adjoint_bin<MS>(V.draws[d], adj[d], S, R, (int)(bin - __ldg(V.bStart + d)), split > 1 ? (int)(item % split) : -1, n);
    }
    flush_adjoint_counters(B.counters, n);
}
