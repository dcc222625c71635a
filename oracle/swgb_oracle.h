/*
 * swgb_oracle.h -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of SwiftShader's triangle draw path, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / --impl reference
 * legs to check and time the GB300 kernels.  Nothing in the swiftshader_gb300
 * package links or calls it.
 *
 * It consumes the same swgb_pipeline_state / swgb_draw_args structs as the
 * C-ABI (include/swgb.h), but every pointer inside them is a HOST pointer.
 */
#ifndef SWGB_ORACLE_H
#define SWGB_ORACLE_H

#include "../include/swgb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Renders one draw into the host attachments of *state.
 * nthreads = 1 runs the reference's semantics in plain primitive order;
 * nthreads > 1 runs the reference's work structure (128-primitive batches set
 * up in parallel, pixels in 16 row-interleaved clusters, primitive order kept
 * per cluster) on that many threads.  Results are identical either way.
 * Counters are accumulated into *cnt when it is non-null. */
swgb_status oracle_draw(const swgb_pipeline_state *state, const swgb_draw_args *args, int nthreads, swgb_counters *cnt);

/* oracle_draw that also records visibility: for every sample plane q and
 * pixel (x, y), the primitives whose fragment passed the depth test, in
 * primitive order.  vis[((q * H + y) * W + x) * visCap + k] holds entry k,
 * visLen[(q * H + y) * W + x] counts every entry (entries past visCap are
 * counted but not stored).  visLen must be zeroed by the caller.  The
 * adjoint's FP64 reference gradient takes its fixed visibility from here. */
swgb_status oracle_draw_visibility(const swgb_pipeline_state *state, const swgb_draw_args *args, int nthreads, swgb_counters *cnt,
                                   uint32_t *vis, uint32_t *visLen, int visCap);

/* 1 in the timing build (FPU flush-to-zero mode instead of the software
 * flush; used only to time the CPU baseline), 0 in the checker build. */
int oracle_timing_build(void);

/* Primitive-level probes, exported so the reference's Reactor known-answer
 * vectors (tests/ReactorUnitTests/ReactorUnitTests.cpp) can pin them. */
int32_t oracle_round_int(float x);         /* RoundInt: cvtss2si, half-even, INT_MIN on overflow */
int32_t oracle_round_int_clamped(float x); /* RoundIntClamped: nearbyint + fptosi.sat            */
int32_t oracle_trunc_int(float x);         /* Int(Float): cvttss2si, INT_MIN on overflow          */
uint16_t oracle_mulhigh_u16(uint16_t a, uint16_t b);
int16_t oracle_mulhigh_s16(int16_t a, int16_t b);
float oracle_fmuladd(float a, float b, float c); /* MulAdd (fused, FTZ/DAZ)                 */
float oracle_log2sqrt(float x);                  /* SamplerCore log2sqrt bit trick        */
float oracle_ftz(float x);

/* Vertex stage probe: transforms one vertex index and returns the Vertex
 * fields the setup stage consumes: out_f[0..3] = clip position,
 * out_f[4] = projected z, out_f[5] = projected w (rhw); out_i[0] = X,
 * out_i[1] = Y, out_i[2] = clipFlags. */
swgb_status oracle_vertex(const swgb_pipeline_state *state, const swgb_draw_args *args, uint32_t vertex_index, float *out_f, int32_t *out_i);

/* Setup stage probe for triangle 'tri' of the draw: returns 1 when the setup
 * routine returns a primitive.  out_i = {yMin, yMax (after trimming), d,
 * clipped}; spans (left, right) for rows [yMin, yMax) written to
 * spans[2*(y-yMin)+0/1] when spans != NULL (capacity 2*max_rows);
 * out_f = {x0, y0, z.A, z.B, z.C, w.A, w.B, w.C, then V[k].A,B,C ...}. */
int oracle_setup(const swgb_pipeline_state *state, const swgb_draw_args *args, uint32_t tri, int32_t *out_i, uint16_t *spans, int max_rows, float *out_f);

/* Samples the pipeline's texture for one 2x2 quad of (u, v) lanes with the
 * implicit LOD, returning 4 lanes x RGBA floats (after getComponentScale),
 * exactly as SamplerCore::sampleTexture128 returns them. */
swgb_status oracle_sample_quad(const swgb_texture *tex, const float u[4], const float v[4], float out[16]);

/* Routine-level probes, compared with SwiftShader's own routines run by
 * oracle/refjit (tests/test_oracle_reference_fixtures.py).
 *
 * oracle_triangle_inputs: what the setup stage receives for triangle tri, in
 * the triangle's setBatchIndices order: vf[3 * 14] (per vertex: clip x, y, z,
 * w, projected z, projected w, 8 varying components, zero past the draw's),
 * vi[3 * 3] (projected X, Y, clip flags), consts = {WxF, HxF, X0xF, Y0xF,
 * depthRange, depthNear}, scissor = {x0, x1, y0, y1}.  Returns the draw's
 * varying component count, or -1.
 *
 * oracle_setup_samples: oracle_setup with every sample's outline:
 * spans[(q * max_rows + r) * 2 + 0/1] = (left, right) of row yMin - 1 + r of
 * sample q for rows yMin - 1 .. yMax, and out_f = {x0, y0, z.A, z.B, z.C, w.A,
 * w.B, w.C, V[k].A, V[k].B, V[k].C ..., zBias}.  Returns visibility, or -1
 * (max_rows too small or invalid state).
 *
 * oracle_set_interpolation_muladd: 1 (default) fuses the mulAdd of
 * QuadRasterizer::interpolate as Reactor's LLVM backend does on an FMA host;
 * 0 lowers it to a multiply and an add, as Reactor's Subzero backend does. */
int oracle_triangle_inputs(const swgb_pipeline_state *state, const swgb_draw_args *args, uint32_t tri, float *vf, int32_t *vi,
                           float *consts, int32_t *scissor);
int oracle_setup_samples(const swgb_pipeline_state *state, const swgb_draw_args *args, uint32_t tri, int32_t *out_i,
                         uint16_t *spans, int max_rows, float *out_f);
void oracle_set_interpolation_muladd(int fused);

#ifdef __cplusplus
}
#endif

#endif
