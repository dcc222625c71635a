/*
 * swgb.h -- C-ABI of the GB300-native draw path (vertex transform + clipping,
 * triangle setup, fixed-point span rasterisation, attribute interpolation,
 * SamplerCore texture filtering, depth test, colour blend/write).
 *
 * This boundary replaces, for the triangle-list FILL path only:
 *   void sw::Renderer::draw(const vk::GraphicsPipeline *, const vk::DynamicState &,
 *                           unsigned count, int baseVertex, CountedEvent *,
 *                           int instanceID, int layer, void *indexBuffer,
 *                           const VkRect2D &renderArea,
 *                           const vk::Pipeline::PushConstantStorage &, bool update)
 *   (src/Device/Renderer.hpp:211-213, body src/Device/Renderer.cpp:183-490)
 * and sw::Renderer::synchronize() (src/Device/Renderer.hpp:218,
 * src/Device/Renderer.cpp:664-671).
 *
 * The vk::GraphicsPipeline state the reference consumes (vk::GraphicsState,
 * src/Device/Context.hpp:443-496; vk::Attachments :112-129; vk::Inputs :132-157;
 * sw::DrawData src/Device/Renderer.hpp:58-113) is flattened into the POD
 * swgb_pipeline_state below.  Enumerants reuse the numeric values of the
 * Vulkan enums they stand for (VkFormat, VkCompareOp, VkBlendFactor, VkBlendOp,
 * VkCullModeFlagBits, VkFrontFace, VkIndexType, VkFilter,
 * VkSamplerMipmapMode, VkSamplerAddressMode), so a Vulkan-side caller copies
 * its create-info fields straight across.
 *
 * All buffer pointers handed to swgb_draw / swgb_draw_batch are DEVICE
 * pointers (cudaMalloc'd, this process, the context's device).  The caller owns
 * them.  The library owns only its scratch memory (post-transform vertices,
 * per-triangle records, bin lists), sized on demand inside the context.
 *
 * Every entry point returns a swgb_status; none aborts the process.
 */
#ifndef SWGB_H
#define SWGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWGB_ABI_VERSION 7

typedef enum swgb_status {
    SWGB_OK = 0,
    SWGB_UNSUPPORTED_STATE = 1, /* state the GB300 path does not implement (reference: UNSUPPORTED()) */
    SWGB_INVALID_ARG = 2,       /* null pointer, zero-sized attachment, out-of-range enum   */
    SWGB_OOM = 3,               /* scratch allocation failed                                 */
    SWGB_DEVICE_TIMEOUT = 4,    /* a bounded device-side wait gave up                        */
    SWGB_DEVICE_ERROR = 5,      /* a CUDA call failed; swgb_last_error() has the text        */
    SWGB_NO_DEVICE = 6          /* no CUDA device visible                                    */
} swgb_status;

/* --- Vulkan enumerant values used by the path (subset) ------------------ */
/* VkFormat */
#define SWGB_FORMAT_UNDEFINED 0
#define SWGB_FORMAT_R8G8B8A8_UNORM 37
#define SWGB_FORMAT_R8G8B8A8_SRGB 43
#define SWGB_FORMAT_B8G8R8A8_UNORM 44
#define SWGB_FORMAT_B8G8R8A8_SRGB 50
#define SWGB_FORMAT_R16G16B16A16_SFLOAT 97
#define SWGB_FORMAT_R32G32_SFLOAT 103
#define SWGB_FORMAT_R32G32B32A32_SFLOAT 109
#define SWGB_FORMAT_D16_UNORM 124
#define SWGB_FORMAT_D32_SFLOAT 126
#define SWGB_FORMAT_S8_UINT 127
/* VkPrimitiveTopology */
#define SWGB_TOPOLOGY_TRIANGLE_LIST 3
#define SWGB_TOPOLOGY_TRIANGLE_STRIP 4
#define SWGB_TOPOLOGY_TRIANGLE_FAN 5
/* VkIndexType (0xFFFFFFFF = non-indexed draw) */
#define SWGB_INDEX_TYPE_UINT16 0
#define SWGB_INDEX_TYPE_UINT32 1
#define SWGB_INDEX_TYPE_UINT8 1000265000u /* VK_INDEX_TYPE_UINT8_EXT */
#define SWGB_INDEX_TYPE_NONE 0xFFFFFFFFu
/* VkCullModeFlagBits */
#define SWGB_CULL_NONE 0
#define SWGB_CULL_FRONT 1
#define SWGB_CULL_BACK 2
#define SWGB_CULL_FRONT_AND_BACK 3
/* VkFrontFace */
#define SWGB_FRONT_FACE_COUNTER_CLOCKWISE 0
#define SWGB_FRONT_FACE_CLOCKWISE 1
/* VkCompareOp */
#define SWGB_COMPARE_NEVER 0
#define SWGB_COMPARE_LESS 1
#define SWGB_COMPARE_EQUAL 2
#define SWGB_COMPARE_LESS_OR_EQUAL 3
#define SWGB_COMPARE_GREATER 4
#define SWGB_COMPARE_NOT_EQUAL 5
#define SWGB_COMPARE_GREATER_OR_EQUAL 6
#define SWGB_COMPARE_ALWAYS 7
/* VkStencilOp */
#define SWGB_STENCIL_OP_KEEP 0
#define SWGB_STENCIL_OP_ZERO 1
#define SWGB_STENCIL_OP_REPLACE 2
#define SWGB_STENCIL_OP_INCREMENT_AND_CLAMP 3
#define SWGB_STENCIL_OP_DECREMENT_AND_CLAMP 4
#define SWGB_STENCIL_OP_INVERT 5
#define SWGB_STENCIL_OP_INCREMENT_AND_WRAP 6
#define SWGB_STENCIL_OP_DECREMENT_AND_WRAP 7
/* VkBlendFactor */
#define SWGB_BLEND_ZERO 0
#define SWGB_BLEND_ONE 1
#define SWGB_BLEND_SRC_COLOR 2
#define SWGB_BLEND_ONE_MINUS_SRC_COLOR 3
#define SWGB_BLEND_DST_COLOR 4
#define SWGB_BLEND_ONE_MINUS_DST_COLOR 5
#define SWGB_BLEND_SRC_ALPHA 6
#define SWGB_BLEND_ONE_MINUS_SRC_ALPHA 7
#define SWGB_BLEND_DST_ALPHA 8
#define SWGB_BLEND_ONE_MINUS_DST_ALPHA 9
/* VkBlendOp */
#define SWGB_BLEND_OP_ADD 0
#define SWGB_BLEND_OP_SUBTRACT 1
#define SWGB_BLEND_OP_REVERSE_SUBTRACT 2
#define SWGB_BLEND_OP_MIN 3
#define SWGB_BLEND_OP_MAX 4
/* VkFilter / VkSamplerMipmapMode / VkSamplerAddressMode */
#define SWGB_FILTER_NEAREST 0
#define SWGB_FILTER_LINEAR 1
#define SWGB_MIPMAP_MODE_NEAREST 0
#define SWGB_MIPMAP_MODE_LINEAR 1
#define SWGB_ADDRESS_REPEAT 0
#define SWGB_ADDRESS_MIRRORED_REPEAT 1
#define SWGB_ADDRESS_CLAMP_TO_EDGE 2
#define SWGB_ADDRESS_CLAMP_TO_BORDER 3
#define SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE 4 /* ADDRESSING_MIRRORONCE */
/* VkBorderColor (the float ones; the integer ones belong to integer formats) */
#define SWGB_BORDER_COLOR_FLOAT_TRANSPARENT_BLACK 0
#define SWGB_BORDER_COLOR_FLOAT_OPAQUE_BLACK 2
#define SWGB_BORDER_COLOR_FLOAT_OPAQUE_WHITE 4
#define SWGB_BORDER_COLOR_FLOAT_CUSTOM_EXT 1000287003u

/* The fixed shaders the path runs in place of SPIR-V modules.
 * VS_MVP_PASSTHROUGH: gl_Position = mvp * attribute[0] (OpMatrixTimesVector,
 *   src/Pipeline/SpirvShaderArithmetic.cpp:39-55); output location k = input
 *   attribute k+1 unchanged.
 * FS_VCOLOR:          outColor = in[0]                       (vec4 colour)
 * FS_TEX_X_VCOLOR:    outColor = texture(tex, in[1].xy) * in[0] (OpFMul) */
#define SWGB_VS_MVP_PASSTHROUGH 1
#define SWGB_FS_VCOLOR 1
#define SWGB_FS_TEX_X_VCOLOR 2

/* Precision profiles of the reference (src/Vulkan/VkConfig.hpp:23-24,101-103).
 * Only the standalone CMake profile (8 sub-pixel bits, fused mulAdd, 16-bit
 * UNORM8 filtering) is implemented; the GN/Chromium legacy profile returns
 * SWGB_UNSUPPORTED_STATE. */
#define SWGB_PRECISION_CMAKE 0
#define SWGB_PRECISION_LEGACY 1

#define SWGB_MAX_ATTRIBS 4
#define SWGB_MAX_MIP_LEVELS 15 /* sw::MIPMAP_LEVELS, src/Device/Config.hpp:23 */

typedef struct swgb_vertex_attrib {
    uint32_t format;   /* R32G32B32A32_SFLOAT or R32G32_SFLOAT                  */
    uint32_t binding;  /* index into swgb_pipeline_state.bindings               */
    uint32_t offset;   /* byte offset of the attribute inside one vertex        */
    uint32_t reserved;
} swgb_vertex_attrib;

typedef struct swgb_vertex_binding {
    const void *buffer; /* device pointer to vertex 0                           */
    uint32_t stride;    /* bytes between consecutive vertices                   */
    uint32_t reserved;
} swgb_vertex_binding;

typedef struct swgb_texture_level {
    const void *buffer;    /* device pointer to texel (0,0) of this level        */
    uint32_t width;
    uint32_t height;
    uint32_t pitch_texels; /* row pitch in texels (Mipmap::pitchP)               */
    uint32_t reserved;
} swgb_texture_level;

/* A combined image sampler (VkDescriptorImageInfo + VkSamplerCreateInfo
 * subset).  Level i of levels[] is image-view level i; entries past
 * level_count are ignored (the descriptor replicates the last level,
 * src/Vulkan/VkDescriptorSetLayout.cpp:468-470). */
typedef struct swgb_texture {
    uint32_t format;      /* R8G8B8A8_UNORM / _SRGB, B8G8R8A8_UNORM / _SRGB, R16G16B16A16_SFLOAT or R32G32B32A32_SFLOAT */
    uint32_t level_count;
    swgb_texture_level levels[SWGB_MAX_MIP_LEVELS];
    uint32_t mag_filter, min_filter, mipmap_mode;
    uint32_t address_u, address_v;
    float mip_lod_bias, min_lod, max_lod;
    uint32_t border_color;          /* SWGB_BORDER_COLOR_*: texels outside a CLAMP_TO_BORDER axis */
    float custom_border_color[4];   /* VkSamplerCustomBorderColorCreateInfoEXT.float32 */
} swgb_texture;

/* VkStencilOpState */
typedef struct swgb_stencil_op_state {
    uint32_t fail_op, pass_op, depth_fail_op, compare_op; /* VkStencilOp x3, VkCompareOp */
    uint32_t compare_mask, write_mask, reference;
    uint32_t reserved;
} swgb_stencil_op_state;

typedef struct swgb_pipeline_state {
    /* vertex input interface (vk::VertexInputInterfaceState): triangle list,
     * strip or fan, provoking vertex first (Renderer.cpp setBatchIndices);
     * primitive restart is resolved by the caller into separate draws, as
     * vk::IndexBuffer does before Renderer::draw */
    uint32_t topology;
    uint32_t attrib_count;
    swgb_vertex_attrib attribs[SWGB_MAX_ATTRIBS];
    swgb_vertex_binding bindings[SWGB_MAX_ATTRIBS];
    /* shaders + push constants */
    uint32_t vertex_shader;
    uint32_t fragment_shader;
    float mvp[16]; /* column-major, the push-constant block of the fixed VS */
    /* pre-rasterization (vk::PreRasterizationState) */
    float viewport_x, viewport_y, viewport_width, viewport_height;
    float viewport_min_depth, viewport_max_depth;
    int32_t scissor_x, scissor_y;
    uint32_t scissor_width, scissor_height;
    uint32_t cull_mode, front_face;
    uint32_t depth_clip_enable;  /* VK_EXT_depth_clip_enable; default true   */
    uint32_t depth_clamp_enable; /* must be 0                                 */
    /* depth bias (VkPipelineRasterizationStateCreateInfo depthBias*, all 0 when
     * depthBiasEnable is false): constant factor, slope factor, clamp (0 = none) */
    float depth_bias_constant, depth_bias_slope, depth_bias_clamp;
    /* fragment (vk::FragmentState) */
    uint32_t depth_test_enable, depth_write_enable, depth_compare_op;
    /* fragment output interface (vk::FragmentOutputInterfaceState) */
    uint32_t color_format;  /* R8G8B8A8_UNORM / _SRGB, B8G8R8A8_UNORM / _SRGB, R16G16B16A16_SFLOAT or R32G32B32A32_SFLOAT */
    uint32_t blend_enable;
    uint32_t src_color_factor, dst_color_factor, color_blend_op;
    uint32_t src_alpha_factor, dst_alpha_factor, alpha_blend_op;
    uint32_t color_write_mask; /* VkColorComponentFlags, 0xF = RGBA        */
    uint32_t sample_count;     /* 1, or 4 (4x MSAA, standard sample locations) */
    /* attachments (vk::Attachments -> DrawData colorBuffer/depthBuffer) */
    void *color;
    uint32_t color_pitch_bytes;
    uint32_t reserved0;
    uint64_t color_slice_bytes;
    void *depth;
    uint32_t depth_pitch_bytes;
    uint32_t depth_format;  /* D32_SFLOAT (or 0, the same) or D16_UNORM */
    uint64_t depth_slice_bytes;
    uint32_t framebuffer_width, framebuffer_height;
    /* the fragment shader's combined image sampler (FS_TEX_X_VCOLOR) */
    swgb_texture texture;
    uint32_t precision_profile;
    /* VkProvokingVertexModeEXT (VK_EXT_provoking_vertex): 0 = FIRST_VERTEX,
     * 1 = LAST_VERTEX; the order setBatchIndices gives each triangle's
     * vertices (src/Device/Renderer.cpp:49-145) */
    uint32_t provoking_vertex;
    /* depth bounds test (VkPipelineDepthStencilStateCreateInfo): the stored
     * depth of a sample must lie in [min_depth_bounds, max_depth_bounds] */
    uint32_t depth_bounds_test_enable;
    float min_depth_bounds, max_depth_bounds;
    /* stencil test (VkPipelineDepthStencilStateCreateInfo) on an S8_UINT
     * attachment: pitch and sample-plane slice in bytes; 'front' applies to
     * front-facing triangles, 'back' to back-facing ones */
    uint32_t stencil_test_enable;
    void *stencil;
    uint32_t stencil_pitch_bytes;
    uint32_t reserved3;
    uint64_t stencil_slice_bytes;
    swgb_stencil_op_state front, back;
} swgb_pipeline_state;

/* The per-draw arguments of sw::Renderer::draw. */
typedef struct swgb_draw_args {
    uint32_t count;        /* number of triangles (Renderer::draw 'count')              */
    int32_t base_vertex;   /* added to every vertex index ('baseVertex')                */
    uint32_t first_vertex; /* non-indexed draws: index of the first vertex              */
    uint32_t index_type;   /* SWGB_INDEX_TYPE_UINT8/16/32, or SWGB_INDEX_TYPE_NONE      */
    const void *indices;   /* device pointer to the first index of the draw             */
    uint32_t vertex_count; /* indexed draws: vertices addressable after base_vertex;
                              every index must be < vertex_count                       */
    int32_t instance_id, layer;
    int32_t render_area_x, render_area_y;
    uint32_t render_area_width, render_area_height;
    /* Primitive restart (VkPipelineInputAssemblyStateCreateInfo::
     * primitiveRestartEnable) of an indexed draw: when nonzero, the draw reads
     * this many indices, and every index equal to the all-ones value of the
     * index type ends a sub-draw, as vk::IndexBuffer::getIndexBuffers splits
     * the index buffer before Renderer::draw (src/Device/Context.cpp:49-91,
     * 249-289); count is then ignored.  The split runs on the device.  Only
     * swgb_draw takes it; swgb_draw_batch and swgb_draw_noalloc return
     * SWGB_UNSUPPORTED_STATE.  0: no restart, count triangles. */
    uint32_t restart_index_count;
    /* Optional cudaEvent_t the caller records on another stream after the
     * last write the draw's texture levels depend on (an upload, a mip-chain
     * blit): the draw waits for it (cudaStreamWaitEvent on the context's
     * stream) only before its raster stage, so vertex processing, setup and
     * binning run while the textures arrive.  NULL: no wait.  swgb_draw_batch
     * and swgb_draw_noalloc wait for it before their first kernel. */
    void *raster_wait_event;
} swgb_draw_args;

/* Device-side counters of one draw (the reference keeps occlusion counts per
 * cluster, src/Device/Renderer.cpp:413-419,524-531).  Accumulated across
 * draws until swgb_reset_counters. */
typedef struct swgb_counters {
    uint64_t triangles_in;       /* triangles submitted                               */
    uint64_t triangles_rejected; /* trivially rejected, clipped away or culled        */
    uint64_t triangles_clipped;  /* triangles that went through the clipper           */
    uint64_t triangles_visible;  /* setup returned a primitive (SetupRoutine 'Return(1)') */
    uint64_t quads;              /* 2x2 quads with non-empty coverage that were shaded */
    uint64_t fragments_tested;   /* covered samples that reached the depth test       */
    uint64_t fragments_passed;   /* samples that passed and were written              */
    uint64_t texture_levels_mask; /* bit i set: mip level i was sampled (OR across draws) */
    /* adjoint (swgb_draw_adjoint*) */
    uint64_t adjoint_fragments;       /* (pixel, primitive) shading adjoints evaluated       */
    uint64_t adjoint_depth_mismatch;  /* samples whose replayed depth differs from the saved depth */
    uint64_t adjoint_list_overflow;   /* blended fragments dropped: more than 2048 on one pixel */
    uint64_t reserved;
} swgb_counters;

typedef struct swgb_ctx swgb_ctx;

/* Library / context management. 'stream' is a cudaStream_t: NULL makes the
 * context create its own non-blocking stream; pass cudaStreamLegacy
 * ((void *)1) to order draws on the legacy default stream. */
int swgb_abi_version(void);
const char *swgb_last_error(void);
swgb_status swgb_ctx_create(int device, void *stream, swgb_ctx **out);
swgb_status swgb_ctx_destroy(swgb_ctx *ctx);
swgb_status swgb_ctx_set_stream(swgb_ctx *ctx, void *stream);

/* Validates and bakes the pipeline state, then enqueues one draw on the
 * context's stream.  Returns before the draw completes (Renderer::draw also
 * returns before its marl tasks finish). */
swgb_status swgb_draw(swgb_ctx *ctx, const swgb_pipeline_state *state, const swgb_draw_args *args);

/* N draws enqueued as batches: the draws' vertex blocks, triangle blocks and
 * screen bins form one work space for one persistent launch of each kernel,
 * replayed from a captured CUDA graph.  The result equals N sequential
 * swgb_draw calls: draws are split into consecutive segments (one graph replay
 * each) wherever a draw touches attachment bytes an earlier draw of the
 * segment touches, or needs another raster variant (colour format or sample
 * count).  Textures and vertex/index buffers must not alias attachments
 * written in the same call. */
swgb_status swgb_draw_batch(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n);

/* The segments swgb_draw_batch would split these draws into, computed on the
 * host without a device: *segment_count segments; when segment_first is not
 * NULL it receives the index (into states/args) of each segment's first draw
 * (room for n entries).  Draws with count 0 belong to no segment. */
swgb_status swgb_plan_batch(const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n, uint32_t *segment_first,
                            uint32_t *segment_count);

/* Allocation-free draw.  No counterpart in the reference: it exists for
 * callers of this library that cannot allocate device memory when they draw --
 * code recording into a CUDA stream capture (cudaMalloc is not capturable), a
 * host whose device memory belongs to another allocator, or a real-time loop
 * that must not enter the allocator.  It runs the same kernels as swgb_draw on
 * 'stream' (a cudaStream_t; NULL = the legacy default stream) on the current
 * device, with all scratch taken from one fixed __device__ array of about
 * 17.3 MiB that every GPU loading this library holds until the process exits.
 * Limits: at most SWGB_NOALLOC_MAX_TRIANGLES triangles and
 * SWGB_NOALLOC_MAX_VERTICES transformed vertices per call; larger draws return
 * SWGB_INVALID_ARG.  The first call on a device resolves the array's device
 * address, so make it before any stream capture begins.  Every call shares
 * the one array: calls whose work overlaps on the GPU (different streams, or
 * several host threads) race and corrupt each other; order them on one stream.
 * Device-side errors (an index >= vertex_count) drop the triangle silently,
 * as there is no context to report them through.  The array's address is
 * resolved once per device and kept for the life of the process, so a
 * device reset (cudaDeviceReset) followed by more calls is not supported.
 * Unlike swgb_draw, this path does not order the bins heaviest first: the
 * result is the same, a large frame can take longer. */
#define SWGB_NOALLOC_MAX_TRIANGLES 32768u
#define SWGB_NOALLOC_MAX_VERTICES 98304u
swgb_status swgb_draw_noalloc(const swgb_pipeline_state *state, const swgb_draw_args *args, void *stream);

/* Adjoint of a draw.  No counterpart in the reference (it has no backward
 * pass).  Given dL/d(colour attachment) after the draw, it adds to the
 * gradient buffers dL/d(texels), dL/d(vertex attributes) and dL/d(vertex
 * positions), holding visibility fixed:
 *   - visibility is recomputed by replaying the draw's coverage and depth
 *     test from the attachment contents before the draw, which must be the
 *     clear values below (the draw ran on freshly cleared attachments); the
 *     saved depth attachment (state->depth, as the draw left it) is compared
 *     against the replay sample by sample (adjoint_depth_mismatch counts
 *     differences);
 *   - the differentiated colour is the perspective-correct interpolation of
 *     the triangle's vertex attributes at the pixel centre, the fixed
 *     fragment shader, the fp32 texture filter with its level of detail held
 *     constant, and the blend (none, or premultiplied OVER: ONE,
 *     ONE_MINUS_SRC_ALPHA, ADD for colour and alpha), with attachment
 *     rounding taken as the identity and sub-pixel snapping ignored;
 *   - positions receive gradients through the barycentrics only (no edge or
 *     visibility terms); depth gets none.
 * Supported: float colour attachments (R16G16B16A16_SFLOAT,
 * R32G32B32A32_SFLOAT), float textures or none, 1 or 4 samples.  Other
 * states return SWGB_UNSUPPORTED_STATE.  Gradients accumulate with fp32
 * atomics, so their low bits vary from run to run.  A blended pixel may hold
 * any number of passing fragments up to 2048 (the excess is counted in
 * adjoint_list_overflow).  The context keeps about 110 KiB of adjoint scratch
 * per resident adjoint warp, allocated on the first adjoint call. */
typedef struct swgb_adjoint_args {
    const float *grad_color;         /* dL/dcolour: float RGBA per pixel and sample, device memory */
    uint32_t grad_color_pitch_bytes; /* row pitch of grad_color                                     */
    uint32_t reserved0;
    uint64_t grad_color_slice_bytes; /* bytes between sample planes of grad_color                   */
    float clear_color[4];            /* attachment contents before the draw                         */
    float clear_depth;
    uint32_t reserved1;
    /* outputs (added to): per mip level, float RGBA per texel with the
     * level's pitch_texels; per vertex binding, a buffer with that binding's
     * stride whose float fields at each attribute's offset receive the
     * attribute's gradient (attribute 0: object-space position) */
    float *grad_texels[SWGB_MAX_MIP_LEVELS];
    void *grad_vertices[SWGB_MAX_ATTRIBS];
} swgb_adjoint_args;
swgb_status swgb_draw_adjoint(swgb_ctx *ctx, const swgb_pipeline_state *state, const swgb_draw_args *args,
                              const swgb_adjoint_args *adj);

/* Adjoints of n independent draws (e.g. views of one scene) as one launch of
 * each kernel: gradients of all draws accumulate into their buffers (which
 * may be shared between draws). */
swgb_status swgb_draw_adjoint_batch(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args,
                                    const swgb_adjoint_args *adjs, uint32_t n);

/* Raster configuration of a context.  No counterpart in the reference, whose
 * work split is fixed (128-primitive batches, 16 row-interleaved clusters,
 * src/Device/Renderer.cpp:551-662, src/Device/Config.hpp).  It chooses how
 * swgb_draw and swgb_draw_batch tile the framebuffer; every configuration
 * gives the same attachments and counters bit for bit.
 *   bin_width x bin_height: the screen bin one raster warp owns, one of
 *     16x16 (default), 32x16, 32x32.  Four-sample draws and draws with a
 *     D16_UNORM depth attachment always use 16x16.
 *   hiz: 1 (default) rejects a triangle's fragments in a bin without
 *     expanding them when the bin's depth bound proves every one fails a
 *     LESS / LESS_OR_EQUAL / GREATER / GREATER_OR_EQUAL test; 0 expands them. */
typedef struct swgb_raster_config {
    uint32_t bin_width;
    uint32_t bin_height;
    uint32_t hiz;
    uint32_t reserved;
} swgb_raster_config;
swgb_status swgb_ctx_set_raster_config(swgb_ctx *ctx, const swgb_raster_config *config);
swgb_status swgb_ctx_get_raster_config(swgb_ctx *ctx, swgb_raster_config *config);

/* Autotuner of the raster configuration.  No counterpart in the reference.
 * It runs the n draws (one swgb_draw_batch when batched != 0, else one
 * swgb_draw each) under every candidate configuration -- each supported bin
 * shape, with hiz on and off -- one untimed warm-up run and then `runs` runs
 * (0 = SWGB_AUTOTUNE_DEFAULT_RUNS; at most SWGB_AUTOTUNE_MAX_RUNS), each
 * timed alone with CUDA events on the context's stream, and sets the
 * context's configuration to the candidate with the lowest median.  The
 * attachment bytes the draws can touch are copied to a temporary device
 * buffer first and restored before every run, so on return the attachments
 * hold the draws' result exactly once (as one swgb_draw_batch / n swgb_draw
 * calls would leave them).  The temporary buffer is as large as those
 * attachment bytes; it is freed before returning.  ms[], ms_min[] and
 * ms_max[] (room for SWGB_AUTOTUNE_CANDIDATES entries each, any may be NULL)
 * receive each candidate's median, fastest and slowest run, and
 * candidates[] (may be NULL) the candidates, in the same order.
 * Synchronises the context's stream. */
#define SWGB_AUTOTUNE_CANDIDATES 6
#define SWGB_AUTOTUNE_DEFAULT_RUNS 3
#define SWGB_AUTOTUNE_MAX_RUNS 15
swgb_status swgb_autotune(swgb_ctx *ctx, const swgb_pipeline_state *states, const swgb_draw_args *args, uint32_t n,
                          int batched, uint32_t runs, swgb_raster_config *best, swgb_raster_config *candidates,
                          double *ms, double *ms_min, double *ms_max);

/* --- The Blitter steps either side of a draw: clears, multisample resolves
 * and scaled blits (mip generation is one LINEAR blit per level), for the
 * attachment and texture formats of the draw path (sw::Blitter,
 * src/Device/Blitter.hpp:144-147, src/Device/Blitter.cpp).  Enqueued on the
 * context's stream like draws; images are device memory. ------------------- */

/* One level and layer of an image (a vk::Image subresource): the first sample
 * plane, its VkFormat, extent, sample count, row pitch (rowPitchBytes) and
 * sample-plane pitch (slicePitchBytes).  data and pitch_bytes must be
 * multiples of the texel size. */
typedef struct swgb_image {
    void *data;
    uint32_t format;
    uint32_t width;
    uint32_t height;
    uint32_t samples; /* 1 or 4 */
    uint64_t pitch_bytes;
    uint64_t slice_bytes;
} swgb_image;

/* VkRect2D */
typedef struct swgb_rect {
    int32_t x, y;
    uint32_t width, height;
} swgb_rect;

/* Blitter::clear (Blitter.cpp:55-168; fastClear :170-300): fills `area` (NULL:
 * the whole image) of every sample plane of dst.  value is given in
 * value_format: R32G32B32A32_SFLOAT (VkClearColorValue.float32[4]) for colour
 * images, D32_SFLOAT (VkClearDepthStencilValue.depth) for D32_SFLOAT and
 * D16_UNORM images, S8_UINT (VkClearDepthStencilValue.stencil, a uint32) for
 * S8_UINT stencil planes.  Normalized formats clamp the value to [0, 1]. */
swgb_status swgb_clear(swgb_ctx *ctx, const void *value, uint32_t value_format, const swgb_image *dst, const swgb_rect *area);

/* VkImageResolve (2D, one layer) */
typedef struct swgb_resolve_region {
    int32_t src_x, src_y;
    int32_t dst_x, dst_y;
    uint32_t width, height;
} swgb_resolve_region;

/* Blitter::resolve (Blitter.cpp:2035-2205): averages the 4 samples of src into
 * the single-sample dst of the same colour format; region NULL = the whole
 * image.  A whole-image resolve of R8G8B8A8_UNORM / B8G8R8A8_UNORM takes the
 * reference's byte-averaging fast path, everything else its float blit. */
swgb_status swgb_resolve(swgb_ctx *ctx, const swgb_image *src, const swgb_image *dst, const swgb_resolve_region *region);

/* VkImageBlit (2D, one layer): two corners {x0, y0, x1, y1} per image; dst
 * corners in reverse order mirror the copy. */
typedef struct swgb_blit_region {
    int32_t src[4];
    int32_t dst[4];
} swgb_blit_region;

/* Blitter::blit (Blitter.cpp:1497-1657,1659-1790,1820-1950): scaled copy of a
 * single-sample colour image box to another, filter SWGB_FILTER_NEAREST or
 * SWGB_FILTER_LINEAR, with the reference's sRGB conversions when the two
 * formats differ in encoding or the copy filters.  The dst box must lie in
 * dst; a src box reaching outside src clamps to its edge. */
swgb_status swgb_blit(swgb_ctx *ctx, const swgb_image *src, const swgb_image *dst, const swgb_blit_region *region, uint32_t filter);

/* Waits for every draw enqueued so far (Renderer::synchronize). */
swgb_status swgb_sync(swgb_ctx *ctx);

/* Counters: copies the device counters to *out (synchronises the stream). */
swgb_status swgb_get_counters(swgb_ctx *ctx, swgb_counters *out);
swgb_status swgb_reset_counters(swgb_ctx *ctx);

/* Number of kernel launches this context has issued since creation. */
uint64_t swgb_launch_count(swgb_ctx *ctx);

/* Kernel timing for benchmarks: with enable = 1 the context records a CUDA
 * event pair on its stream around every kernel launch; with enable =
 * SWGB_KERNEL_TIMING_KINDS(mask) only around launches of the kinds whose bit
 * (1 << SWGB_KERNEL_*) is in mask (each pair costs the stream a little time).
 * swgb_get_kernel_times synchronises, sums the elapsed milliseconds per kernel
 * kind (SWGB_KERNEL_*) into ms[] and the launch counts into launches[], then
 * forgets the recorded pairs. */
#define SWGB_KERNEL_TIMING_KINDS(mask) (0x10000 | ((mask) & 0xFFFF))
#define SWGB_KERNEL_VERTEX 0
#define SWGB_KERNEL_SETUP 1
#define SWGB_KERNEL_RASTER 2
#define SWGB_KERNEL_BATCH 3 /* one graph replay of a batch segment (three kernels) */
#define SWGB_KERNEL_ADJOINT 4
#define SWGB_KERNEL_BIN_ORDER 5 /* binning of a single draw: bin order and bin lists */
#define SWGB_KERNEL_BLIT 6      /* swgb_clear / swgb_resolve / swgb_blit */
#define SWGB_KERNEL_KINDS 8
swgb_status swgb_set_kernel_timing(swgb_ctx *ctx, int enable);
swgb_status swgb_get_kernel_times(swgb_ctx *ctx, double ms[SWGB_KERNEL_KINDS], uint32_t launches[SWGB_KERNEL_KINDS]);

#ifdef __cplusplus
}
#endif

#endif /* SWGB_H */
