/*
 * refjit_harness.cpp -- TEST INFRASTRUCTURE ONLY (never part of the product).
 *
 * Drives SwiftShader's own draw routines, compiled from the reference sources
 * by oracle/refjit/build_refjit.py, directly on the host CPU (no Vulkan entry
 * point, ICD or loader), so the oracle's restatement of them can be pinned to
 * the reference itself:
 *
 *   refjit_setup       Clipper::Clip (src/Device/Clipper.cpp:22-299) and the
 *                      JIT-compiled SetupRoutine (src/Pipeline/SetupRoutine.cpp:36-621)
 *                      for one triangle: y range, per-sample outline spans,
 *                      x0/y0, z/w/varying plane equations and zBias;
 *   refjit_sample_quad a SamplerCore routine wrapped as SpirvEmitter::
 *                      emitSamplerRoutine wraps it (src/Pipeline/SpirvShaderSampling.cpp:153-273),
 *                      implicit LOD, one 2x2 quad of coordinates;
 *   refjit_raster      setup of every triangle of a draw, then the JIT-compiled
 *                      QuadRasterizer + PixelRoutine (src/Device/QuadRasterizer.cpp:71-233,
 *                      src/Pipeline/PixelRoutine.cpp) of a pipeline without a
 *                      fragment shader (spirvShader == nullptr: coverage, depth
 *                      bias, depth clamp, depth bounds, stencil, depth test and
 *                      write, occlusion count), one cluster, primitive order;
 *                      counts[] = {visible, clipped, occlusion samples,
 *                      nanoseconds of the setup loop, of the pixel routine}.
 *
 * The vertex stage (VertexRoutine + the MVP shader) and the draw constants
 * (Renderer::draw) stay the oracle's: the caller passes the oracle's vertex
 * records and constants in, so each comparison isolates one reference routine.
 * The glue this file restates (the fields SetupProcessor::update,
 * PixelProcessor::update and Renderer::draw put into the routines' state and
 * DrawData, and the loop of DrawCall::setupSolidTriangles) cites its lines.
 *
 * Routines run with FTZ/DAZ set, as the reference's worker threads run them
 * (src/System/SwiftConfig.cpp:136-139).  x86-64 only (the Subzero backend built
 * for this harness).
 */
#include "Device/Clipper.hpp"
#include "Device/Polygon.hpp"
#include "Device/Primitive.hpp"
#include "Device/Renderer.hpp"
#include "Device/Sampler.hpp"
#include "Device/Vertex.hpp"
#include "Pipeline/Constants.hpp"
#include "Pipeline/PixelProgram.hpp"
#include "Pipeline/SamplerCore.hpp"
#include "Pipeline/SetupRoutine.hpp"
#include "Vulkan/VkDevice.hpp"

#include "swgb.h"

#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#if defined(__x86_64__)
#include <xmmintrin.h>
#endif

using namespace rr;

namespace {

constexpr int kMaxV = 8;  // varying components of the fixed shaders (vColor + uv)

// Storage laid out as a vk::Device whose only initialised member is the
// sw::Constants the routines read through `device + OFFSET(vk::Device, constants)`.
struct Env
{
	unsigned char *device = nullptr;
	Env()
	{
		device = static_cast<unsigned char *>(std::aligned_alloc(64, (sizeof(vk::Device) + 63) & ~size_t(63)));
		std::memset(device, 0, sizeof(vk::Device));
		new(device + OFFSET(vk::Device, constants)) sw::Constants();
	}
	const vk::Device *dev() const { return reinterpret_cast<const vk::Device *>(device); }
	const sw::Constants *constants() const { return reinterpret_cast<const sw::Constants *>(device + OFFSET(vk::Device, constants)); }
};

Env &env()
{
	static Env e;
	return e;
}

std::mutex g_mutex;

struct FtzDaz
{
#if defined(__x86_64__)
	unsigned int saved;
	FtzDaz()
	    : saved(_mm_getcsr())
	{
		_mm_setcsr(saved | 0x8040);  // FTZ | DAZ
	}
	~FtzDaz() { _mm_setcsr(saved); }
#endif
};

// Input record of one vertex (the oracle's vertex-stage output).
// vf: clip x, y, z, w, projected z, projected w, varyings[kMaxV]
// vi: projected X, projected Y, clip flags
constexpr int kVF = 6 + kMaxV;
constexpr int kVI = 3;

void fill_vertex(sw::Vertex &v, const float *vf, const int32_t *vi, int nv)
{
	std::memset(&v, 0, sizeof(v));
	v.x = vf[0];
	v.y = vf[1];
	v.z = vf[2];
	v.w = vf[3];
	v.projected.z = vf[4];
	v.projected.w = vf[5];
	v.projected.x = vi[0];
	v.projected.y = vi[1];
	v.clipFlags = vi[2];
	v.cullMask = 0xF;  // the fixed VS writes no cull distances
	for(int k = 0; k < nv; k++) v.v[k] = vf[6 + k];
}

// consts: WxF, HxF, X0xF, Y0xF, depthRange, depthNear (Renderer.cpp:300-331);
// scissor: x0, x1, y0, y1 after the render-area clamp (Renderer.cpp:333-345).
void fill_draw_data(sw::DrawData &d, const swgb_pipeline_state *st, const float *consts, const int32_t *scissor)
{
	d.WxF = consts[0];
	d.HxF = consts[1];
	d.X0xF = consts[2];
	d.Y0xF = consts[3];
	d.depthRange = consts[4];
	d.depthNear = consts[5];
	d.constantDepthBias = st->depth_bias_constant;  // Renderer.cpp:321-323
	d.slopeDepthBias = st->depth_bias_slope;
	// PreRasterizationState::getDepthBiasClamp keeps a NaN clamp out (Context.cpp:650-661)
	d.depthBiasClamp = (st->depth_bias_clamp == st->depth_bias_clamp) ? st->depth_bias_clamp : 0.0f;
	d.minimumResolvableDepthDifference = (st->depth_format == SWGB_FORMAT_D16_UNORM) ? 1.01f / 0xFFFF : 0.0f;  // Renderer.cpp:424-438
	d.scissorX0 = scissor[0];
	d.scissorX1 = scissor[1];
	d.scissorY0 = scissor[2];
	d.scissorY1 = scissor[3];
}

// SetupProcessor::update (src/Device/SetupProcessor.cpp:58-103) for the
// fixed shaders: triangles, every varying component smooth (perspective).
sw::SetupProcessor::State setup_state(const swgb_pipeline_state *st, int nv, bool fragmentShader)
{
	sw::SetupProcessor::State s;
	s.isDrawPoint = false;
	s.isDrawLine = false;
	s.isDrawTriangle = true;
	s.fixedPointDepthBuffer = st->depth != nullptr && st->depth_format == SWGB_FORMAT_D16_UNORM;
	s.applyConstantDepthBias = st->depth_bias_constant != 0.0f;
	s.applySlopeDepthBias = st->depth_bias_slope != 0.0f;
	s.applyDepthBiasClamp = st->depth_bias_clamp != 0.0f;
	s.interpolateZ = st->depth != nullptr && st->depth_test_enable;
	s.interpolateW = fragmentShader;
	s.frontFace = st->front_face == SWGB_FRONT_FACE_CLOCKWISE ? VK_FRONT_FACE_CLOCKWISE : VK_FRONT_FACE_COUNTER_CLOCKWISE;
	s.cullMode = st->cull_mode;
	s.multiSampleCount = st->sample_count;
	s.enableMultiSampling = st->sample_count > 1;
	s.numClipDistances = 0;
	s.numCullDistances = 0;
	if(fragmentShader)
	{
		for(int k = 0; k < nv; k++)
		{
			s.gradient[k].Type = sw::SpirvShader::ATTRIBTYPE_FLOAT;
			s.gradient[k].Flat = false;
			s.gradient[k].Centroid = false;
			s.gradient[k].NoPerspective = false;
		}
	}
	s.hash = 0;  // only the routine caches read it
	return s;
}

std::string key_of(const void *p, size_t n)
{
	return std::string(static_cast<const char *>(p), n);
}

// JIT-compiled routines, kept per state (as the reference's routine caches do).
std::map<std::string, sw::SetupFunction::RoutineType> g_setup;
std::map<std::string, sw::RasterizerFunction::RoutineType> g_raster;
std::map<std::string, std::shared_ptr<rr::Routine>> g_sampler;
std::vector<std::unique_ptr<sw::PixelProcessor::State>> g_pixelStates;

sw::SetupFunction::RoutineType setup_routine(const sw::SetupProcessor::State &s)
{
	const std::string k = key_of(&s, sizeof(s));
	auto it = g_setup.find(k);
	if(it != g_setup.end()) return it->second;
	sw::SetupRoutine gen(s);
	gen.generate();
	auto r = gen.getRoutine();
	g_setup[k] = r;
	return r;
}

// DrawCall::setupSolidTriangles for one triangle (src/Device/Renderer.cpp:733-776):
// trivial reject, Clipper::Clip, then the setup routine.  prims receives
// sample_count Primitives.  Returns 1 when visible; *clipped is set when the
// triangle went through the clipper.
int setup_one(const sw::SetupFunction::RoutineType &routine, const swgb_pipeline_state *st, sw::DrawData *data,
              sw::DrawCall *call, sw::Triangle *tri, sw::Primitive *prims, int *clipped)
{
	sw::Vertex &v0 = tri->v0, &v1 = tri->v1, &v2 = tri->v2;
	sw::Polygon polygon(&v0.position, &v1.position, &v2.position);
	*clipped = 0;
	if((v0.cullMask | v1.cullMask | v2.cullMask) == 0) return 0;
	if((v0.clipFlags & v1.clipFlags & v2.clipFlags) != sw::Clipper::CLIP_FINITE) return 0;
	const int clipFlagsOr = v0.clipFlags | v1.clipFlags | v2.clipFlags;
	if(clipFlagsOr != sw::Clipper::CLIP_FINITE)
	{
		*clipped = 1;
		if(!sw::Clipper::Clip(polygon, clipFlagsOr, *call)) return 0;
	}
	return routine(env().dev(), prims, tri, &polygon, data);
}

// A DrawCall object only as far as Clipper::Clip reads it (depthClipNegativeOneToOne).
struct CallStorage
{
	alignas(alignof(sw::DrawCall)) unsigned char bytes[sizeof(sw::DrawCall)];
	CallStorage()
	{
		std::memset(bytes, 0, sizeof(bytes));
		reinterpret_cast<sw::DrawCall *>(bytes)->depthClipNegativeOneToOne = false;
	}
	sw::DrawCall *get() { return reinterpret_cast<sw::DrawCall *>(bytes); }
};

vk::Format vk_format(uint32_t f)
{
	return vk::Format(static_cast<VkFormat>(f));
}

VkCompareOp vk_compare(uint32_t op) { return static_cast<VkCompareOp>(op); }

sw::PixelProcessor::States::StencilOpState stencil_state(const swgb_stencil_op_state &s)
{
	VkStencilOpState v = {};
	v.failOp = static_cast<VkStencilOp>(s.fail_op);
	v.passOp = static_cast<VkStencilOp>(s.pass_op);
	v.depthFailOp = static_cast<VkStencilOp>(s.depth_fail_op);
	v.compareOp = vk_compare(s.compare_op);
	v.compareMask = s.compare_mask;
	v.writeMask = s.write_mask;
	v.reference = s.reference;
	sw::PixelProcessor::States::StencilOpState o;
	o = v;
	return o;
}

}  // namespace

extern "C" {

/* Setup of one triangle.  v: three vertex records (vf[kVF], vi[kVI] each, the
 * oracle's vertex-stage output, in the triangle's setBatchIndices order);
 * consts/scissor: the draw constants.  out_i = {yMin, yMax, clipped, visible};
 * spans[(q * max_rows + r) * 2 + 0/1] = (left, right) of row yMin - 1 + r of
 * sample q, for rows yMin - 1 .. yMax (max_rows >= yMax - yMin + 2);
 * out_f = {x0, y0, z.A, z.B, z.C, w.A, w.B, w.C, V[k].A, V[k].B, V[k].C ...,
 * zBias}.  Returns 0, or -1 on bad arguments. */
int refjit_setup(const swgb_pipeline_state *st, const float *consts, const int32_t *scissor, const float *vf,
                 const int32_t *vi, int nv, int32_t *out_i, uint16_t *spans, int max_rows, float *out_f)
{
	if(!st || !consts || !scissor || !vf || !vi || nv < 0 || nv > kMaxV || !out_i) return -1;
	if(st->sample_count != 1 && st->sample_count != 4) return -1;
	std::lock_guard<std::mutex> lock(g_mutex);
	FtzDaz ftz;
	const int ms = st->sample_count;
	auto routine = setup_routine(setup_state(st, nv, true));
	std::unique_ptr<sw::DrawData> data(new sw::DrawData());
	fill_draw_data(*data, st, consts, scissor);
	CallStorage call;
	std::unique_ptr<sw::Triangle> tri(new sw::Triangle());
	fill_vertex(tri->v0, vf + 0 * kVF, vi + 0 * kVI, nv);
	fill_vertex(tri->v1, vf + 1 * kVF, vi + 1 * kVI, nv);
	fill_vertex(tri->v2, vf + 2 * kVF, vi + 2 * kVI, nv);
	std::vector<sw::Primitive> prims(ms);
	std::memset(prims.data(), 0, sizeof(sw::Primitive) * ms);
	int clipped = 0;
	const int vis = setup_one(routine, st, data.get(), call.get(), tri.get(), prims.data(), &clipped);
	const sw::Primitive &p = prims[0];
	out_i[0] = vis ? p.yMin : 0;
	out_i[1] = vis ? p.yMax : 0;
	out_i[2] = clipped;
	out_i[3] = vis;
	if(vis && spans)
	{
		const int rows = p.yMax - p.yMin + 2;
		if(rows > max_rows) return -1;
		for(int q = 0; q < ms; q++)
			for(int r = 0; r < rows; r++)
			{
				const int y = p.yMin - 1 + r;
				spans[(q * max_rows + r) * 2 + 0] = prims[q].outline[y].left;
				spans[(q * max_rows + r) * 2 + 1] = prims[q].outline[y].right;
			}
	}
	if(vis && out_f)
	{
		out_f[0] = p.x0;
		out_f[1] = p.y0;
		out_f[2] = p.z.A;
		out_f[3] = p.z.B;
		out_f[4] = p.z.C;
		out_f[5] = p.w.A;
		out_f[6] = p.w.B;
		out_f[7] = p.w.C;
		for(int k = 0; k < nv; k++)
		{
			out_f[8 + 3 * k + 0] = p.V[k].A;
			out_f[8 + 3 * k + 1] = p.V[k].B;
			out_f[8 + 3 * k + 2] = p.V[k].C;
		}
		out_f[8 + 3 * nv] = p.zBias;
	}
	return 0;
}

/* A SamplerCore routine for the texture and sampler state of *tex (levels are
 * host memory, tightly pitched by pitch_bytes), sampling one 2x2 quad of
 * coordinates with the implicit LOD; out[4 * c + lane] = component c of lane
 * (the routine's SIMD::Float4 output, after getComponentScale).  The
 * descriptor's mip levels past the image's last repeat the last
 * (VkDescriptorSetLayout.cpp:469-503); a single-level image sampled with
 * MIN/MAG filters equal forces minLod = maxLod = 0
 * (SpirvShaderSampling.cpp:92-99).  Returns 0, or -1 on bad arguments. */
int refjit_sample_quad(const swgb_texture *tex, const float *u, const float *v, float *out)
{
	if(!tex || !u || !v || !out || tex->level_count < 1 || tex->level_count > SWGB_MAX_MIP_LEVELS) return -1;
	std::lock_guard<std::mutex> lock(g_mutex);
	FtzDaz ftz;

	sw::Sampler s = {};
	s.textureType = VK_IMAGE_VIEW_TYPE_2D;
	s.textureFormat = vk_format(tex->format);
	auto addressing = [](uint32_t m) {
		switch(m)
		{
		case SWGB_ADDRESS_REPEAT: return sw::ADDRESSING_WRAP;
		case SWGB_ADDRESS_MIRRORED_REPEAT: return sw::ADDRESSING_MIRROR;
		case SWGB_ADDRESS_CLAMP_TO_EDGE: return sw::ADDRESSING_CLAMP;
		case SWGB_ADDRESS_CLAMP_TO_BORDER: return sw::ADDRESSING_BORDER;
		case SWGB_ADDRESS_MIRROR_CLAMP_TO_EDGE: return sw::ADDRESSING_MIRRORONCE;
		default: return sw::ADDRESSING_WRAP;
		}
	};
	s.addressingModeU = addressing(tex->address_u);
	s.addressingModeV = addressing(tex->address_v);
	s.addressingModeW = sw::ADDRESSING_WRAP;
	// convertMipmapMode / convertFilterMode (SpirvShaderSampling.cpp:275-431) for a 2D view, Implicit method
	s.mipmapFilter = tex->mipmap_mode == SWGB_MIPMAP_MODE_LINEAR ? sw::MIPMAP_LINEAR : sw::MIPMAP_POINT;
	if(tex->min_filter == SWGB_FILTER_LINEAR && tex->mag_filter == SWGB_FILTER_LINEAR) s.textureFilter = sw::FILTER_LINEAR;
	else if(tex->min_filter == SWGB_FILTER_NEAREST && tex->mag_filter == SWGB_FILTER_NEAREST) s.textureFilter = sw::FILTER_POINT;
	else if(tex->min_filter == SWGB_FILTER_NEAREST) s.textureFilter = sw::FILTER_MIN_POINT_MAG_LINEAR;
	else s.textureFilter = sw::FILTER_MIN_LINEAR_MAG_POINT;
	s.swizzle = { VK_COMPONENT_SWIZZLE_R, VK_COMPONENT_SWIZZLE_G, VK_COMPONENT_SWIZZLE_B, VK_COMPONENT_SWIZZLE_A };
	s.gatherComponent = 0;
	s.highPrecisionFiltering = false;
	s.compareEnable = false;
	s.border = static_cast<VkBorderColor>(tex->border_color);
	for(int c = 0; c < 4; c++) s.customBorder.float32[c] = tex->custom_border_color[c];
	s.unnormalizedCoordinates = false;
	s.mipLodBias = tex->mip_lod_bias;
	s.maxAnisotropy = 1.0f;
	s.minLod = tex->min_lod;
	s.maxLod = tex->max_lod;
	if(tex->level_count == 1 && s.textureFilter != sw::FILTER_MIN_POINT_MAG_LINEAR && s.textureFilter != sw::FILTER_MIN_LINEAR_MAG_POINT)
	{
		s.minLod = 0.0f;
		s.maxLod = 0.0f;
	}

	const std::string k = key_of(&s, sizeof(s));
	auto it = g_sampler.find(k);
	std::shared_ptr<rr::Routine> routine;
	if(it != g_sampler.end()) routine = it->second;
	else
	{
		rr::Function<Void(Pointer<Byte>, Pointer<SIMD::Float>, Pointer<SIMD::Float>, Pointer<Byte>)> function;
		{
			Pointer<Byte> texture = function.Arg<0>();
			Pointer<SIMD::Float> in = function.Arg<1>();
			Pointer<SIMD::Float> outp = function.Arg<2>();
			Pointer<Byte> constants = function.Arg<3>();
			SIMD::Float uvwa[4];
			uvwa[0] = in[0];
			uvwa[1] = in[1];
			SIMD::Float dRef;
			SIMD::Float dsx, dsy;
			SIMD::Int offset[4];
			SIMD::Int sampleId;
			sw::SamplerFunction fn = { sw::Implicit };
			sw::SamplerCore core(constants, s, fn);
			Float lod = Float(0.0f);  // bias operand of Implicit sampling: none
			sw::SIMD::Float4 r = core.sampleTexture(texture, uvwa, dRef, lod, dsx, dsy, offset, sampleId);
			outp[0] = r.x;
			outp[1] = r.y;
			outp[2] = r.z;
			outp[3] = r.w;
		}
		routine = function("sampler");
		g_sampler[k] = routine;
	}

	// The descriptor's sw::Texture (WriteTextureLevelInfo, VkDescriptorSetLayout.cpp:299-331)
	std::unique_ptr<sw::Texture> t(new sw::Texture());
	std::memset(t.get(), 0, sizeof(sw::Texture));
	const uint32_t bytes = s.textureFormat.bytes();
	for(int level = 0; level < sw::MIPMAP_LEVELS; level++)
	{
		const int l = level < (int)tex->level_count ? level : (int)tex->level_count - 1;
		const swgb_texture_level &lv = tex->levels[l];
		const uint32_t w = lv.width, h = lv.height, pitchP = lv.pitch_texels;
		if(level == 0)
		{
			t->widthWidthHeightHeight = sw::float4((float)w, (float)w, (float)h, (float)h);
			t->width = sw::float4((float)w);
			t->height = sw::float4((float)h);
			t->depth = sw::float4(1.0f);
		}
		sw::Mipmap &m = t->mipmap[level];
		m.buffer = lv.buffer;
		m.uHalf = sw::ushort4((uint16_t)(0x8000 / w));
		m.vHalf = sw::ushort4((uint16_t)(0x8000 / h));
		m.wHalf = sw::ushort4((uint16_t)0x8000);
		m.width = sw::uint4(w);
		m.height = sw::uint4(h);
		m.depth = sw::uint4(1);
		m.onePitchP[0] = 1;
		m.onePitchP[1] = (short)pitchP;
		m.onePitchP[2] = 1;
		m.onePitchP[3] = (short)pitchP;
		m.pitchP = sw::uint4(pitchP);
		m.sliceP = sw::uint4(pitchP * h);
		m.samplePitchP = sw::uint4(pitchP * h);
		m.sampleMax = sw::uint4(0);
	}
	alignas(16) float in[2][4];
	alignas(16) float o[4][4];
	for(int i = 0; i < 4; i++)
	{
		in[0][i] = u[i];
		in[1][i] = v[i];
	}
	auto entry = reinterpret_cast<void (*)(const void *, const void *, void *, const void *)>(const_cast<void *>(routine->getEntry(0)));
	entry(t.get(), in, o, env().constants());
	for(int c = 0; c < 4; c++)
		for(int i = 0; i < 4; i++) out[4 * c + i] = o[c][i];
	return 0;
}

/* One draw's depth / stencil result under the reference's rasteriser and
 * pixel routine without a fragment shader.  vf/vi: 3 * ntri vertex records
 * (triangle t at 3t .. 3t+2), consts/scissor as refjit_setup.  The depth and
 * stencil attachments of *st (host memory, sample planes depth_slice /
 * stencil_slice bytes apart) are updated in place.  counts = {visible
 * triangles, clipped triangles, occlusion samples}.  Returns 0, or -1 on bad
 * arguments. */
int refjit_raster(const swgb_pipeline_state *st, const float *consts, const int32_t *scissor, const float *vf, const int32_t *vi,
                  int ntri, int nv, uint64_t *counts)
{
	if(!st || !consts || !scissor || (ntri && (!vf || !vi)) || !counts) return -1;
	if(st->sample_count != 1 && st->sample_count != 4) return -1;
	if(st->framebuffer_height + 2 > sw::OUTLINE_RESOLUTION) return -1;
	std::lock_guard<std::mutex> lock(g_mutex);
	FtzDaz ftz;
	const int ms = st->sample_count;
	auto sroutine = setup_routine(setup_state(st, nv, false));

	// PixelProcessor::update (src/Device/PixelProcessor.cpp:74-185), no fragment shader
	std::unique_ptr<sw::PixelProcessor::State> ps(new sw::PixelProcessor::State());
	const bool depthAtt = st->depth != nullptr && st->depth_format != SWGB_FORMAT_UNDEFINED;
	const bool stencilAtt = st->stencil != nullptr;
	ps->depthFormat = depthAtt ? vk_format(st->depth_format) : vk::Format(VK_FORMAT_UNDEFINED);
	ps->depthWriteEnable = depthAtt && st->depth_test_enable && st->depth_write_enable;
	if(stencilAtt && st->stencil_test_enable)
	{
		ps->stencilActive = true;
		ps->frontStencil = stencil_state(st->front);
		ps->backStencil = stencil_state(st->back);
	}
	ps->depthBoundsTestActive = depthAtt && st->depth_bounds_test_enable;
	ps->minDepthBounds = st->min_depth_bounds;
	ps->maxDepthBounds = st->max_depth_bounds;
	if(depthAtt && st->depth_test_enable)
	{
		ps->depthTestActive = true;
		ps->depthCompareMode = vk_compare(st->depth_compare_op);
		ps->depthBias = st->depth_bias_constant != 0.0f || st->depth_bias_slope != 0.0f;
		ps->depthClamp = true;  // no VK_EXT_depth_range_unrestricted: [0, 1]
		ps->minDepthClamp = 0.0f;
		ps->maxDepthClamp = 1.0f;
	}
	ps->occlusionEnabled = true;
	for(int i = 0; i < sw::MAX_COLOR_BUFFERS; i++) ps->colorFormat[i] = vk::Format(VK_FORMAT_UNDEFINED);
	ps->colorWriteMask = 0;
	ps->multiSampleCount = ms;
	ps->multiSampleMask = ms > 1 ? 0xF : 0x1;
	ps->enableMultiSampling = ms > 1;
	ps->frontFace = st->front_face == SWGB_FRONT_FACE_CLOCKWISE ? VK_FRONT_FACE_CLOCKWISE : VK_FRONT_FACE_COUNTER_CLOCKWISE;
	ps->hash = 0;

	const std::string k = key_of(ps.get(), sizeof(sw::PixelProcessor::State));
	sw::RasterizerFunction::RoutineType proutine;
	auto it = g_raster.find(k);
	if(it != g_raster.end()) proutine = it->second;
	else
	{
		// the routine keeps a reference to its state: keep the state alive
		g_pixelStates.emplace_back(new sw::PixelProcessor::State(*ps));
		vk::Attachments attachments;
		vk::DescriptorSet::Bindings bindings = {};
		sw::PixelProgram gen(*g_pixelStates.back(), nullptr, nullptr, attachments, bindings);
		gen.generate();
		proutine = gen("PixelRoutine_refjit");
		g_raster[k] = proutine;
	}

	std::unique_ptr<sw::DrawData> data(new sw::DrawData());
	fill_draw_data(*data, st, consts, scissor);
	data->depthBuffer = static_cast<float *>(st->depth);
	data->depthPitchB = (int)st->depth_pitch_bytes;
	data->depthSliceB = (int)st->depth_slice_bytes;
	data->stencilBuffer = static_cast<unsigned char *>(st->stencil);
	data->stencilPitchB = (int)st->stencil_pitch_bytes;
	data->stencilSliceB = (int)st->stencil_slice_bytes;
	data->stencil[0].set(st->front.reference, st->front.compare_mask, st->front.write_mask);  // Renderer.cpp:385-386
	data->stencil[1].set(st->back.reference, st->back.compare_mask, st->back.write_mask);
	data->occlusion[0] = 0;

	CallStorage call;
	std::unique_ptr<sw::Triangle> tri(new sw::Triangle());
	std::vector<sw::Primitive> prims;
	prims.reserve((size_t)ntri * ms);
	std::vector<sw::Primitive> one(ms);
	uint64_t visible = 0, clippedN = 0;
	const auto t0 = std::chrono::steady_clock::now();
	for(int t = 0; t < ntri; t++)
	{
		fill_vertex(tri->v0, vf + (3 * t + 0) * kVF, vi + (3 * t + 0) * kVI, nv);
		fill_vertex(tri->v1, vf + (3 * t + 1) * kVF, vi + (3 * t + 1) * kVI, nv);
		fill_vertex(tri->v2, vf + (3 * t + 2) * kVF, vi + (3 * t + 2) * kVI, nv);
		std::memset(one.data(), 0, sizeof(sw::Primitive) * ms);
		int clipped = 0;
		if(setup_one(sroutine, st, data.get(), call.get(), tri.get(), one.data(), &clipped))
		{
			visible++;
			for(int q = 0; q < ms; q++) prims.push_back(one[q]);
		}
		clippedN += clipped;
	}
	// the pixel routine walks `count` primitives of stride ms * sizeof(Primitive)
	// (QuadRasterizer.cpp:71-100, one cluster covers every row)
	const auto t1 = std::chrono::steady_clock::now();
	if(visible) proutine(env().dev(), prims.data(), (int)visible, 0, 1, data.get());
	const auto t2 = std::chrono::steady_clock::now();
	counts[0] = visible;
	counts[1] = clippedN;
	counts[2] = data->occlusion[0];
	// nanoseconds of the setup loop and of the pixel routine's call
	counts[3] = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count();
	counts[4] = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t2 - t1).count();
	return 0;
}

}  // extern "C"
