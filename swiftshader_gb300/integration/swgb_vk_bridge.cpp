// swgb_vk_bridge.cpp -- the reference-side binding of libswgb: fills the
// C-ABI structs of include/swgb.h from the state SwiftShader's
// sw::Renderer::draw holds (src/Device/Renderer.cpp:183-490), so that
// Renderer::draw can hand a triangle draw to the GB300 path and keep its own
// CPU routines for everything else.
//
// It is written against SwiftShader's headers and is meant to be compiled
// inside the SwiftShader tree (next to src/Device/Renderer.cpp); this
// repository compiles it syntax-only against the reference sources to show
// that every field has a source (tests/test_integration_bridge.py).  It is
// not part of libswgb.
//
// Sources of the fields (src/Device/Context.hpp):
//   VertexInputInterfaceState  topology, primitive restart         (:251-280)
//   PreRasterizationState      viewport, scissor, cull mode, front face,
//                              depth clip / clamp, depth bias, provoking vertex (:282-353)
//   FragmentState              depth test / write / compare op, depth
//                              bounds, stencil                       (:355-400)
//   FragmentOutputInterfaceState  sample count, blend state, write mask (:402-440)
//   Attachments / ImageView    attachment pointers, formats, pitches (:112-129)
//   Inputs / sw::Stream        vertex streams                        (:132-157, Device/Stream.hpp)
//   SampledImageDescriptor / SamplerState  the texture and its sampler
//                              (Vulkan/VkDescriptorSetLayout.hpp:37-52, Vulkan/VkSampler.hpp)
//   push constants             the fixed vertex shader's column-major MVP

#include "Device/Context.hpp"
#include "Device/Renderer.hpp"
#include "Vulkan/VkDescriptorSetLayout.hpp"
#include "Vulkan/VkDevice.hpp"
#include "Vulkan/VkImageView.hpp"
#include "Vulkan/VkPipeline.hpp"
#include "Vulkan/VkSampler.hpp"

#include "swgb.h"

#include <cstring>

namespace swgb_bridge {

namespace {

bool supported_color(VkFormat f)
{
	return f == VK_FORMAT_R8G8B8A8_UNORM || f == VK_FORMAT_R8G8B8A8_SRGB || f == VK_FORMAT_B8G8R8A8_UNORM ||
	       f == VK_FORMAT_B8G8R8A8_SRGB || f == VK_FORMAT_R16G16B16A16_SFLOAT || f == VK_FORMAT_R32G32B32A32_SFLOAT;
}

// vk::FragmentOutputInterfaceState::getBlendState returns the blend state
// after SwiftShader's simplification (Context.cpp:1090-1270), whose operations
// may be its private VK_BLEND_OP_ZERO_EXT / SRC_EXT / DST_EXT; libswgb takes
// Vulkan's own operations and simplifies the same way, so each private
// operation goes back as the standard triple it stands for.
void blend_triple(VkBlendOp op, VkBlendFactor sf, VkBlendFactor df, uint32_t &o, uint32_t &s, uint32_t &d)
{
	switch(op)
	{
	case VK_BLEND_OP_ZERO_EXT: o = SWGB_BLEND_OP_ADD; s = SWGB_BLEND_ZERO; d = SWGB_BLEND_ZERO; return;
	case VK_BLEND_OP_SRC_EXT: o = SWGB_BLEND_OP_ADD; s = SWGB_BLEND_ONE; d = SWGB_BLEND_ZERO; return;
	case VK_BLEND_OP_DST_EXT: o = SWGB_BLEND_OP_ADD; s = SWGB_BLEND_ZERO; d = SWGB_BLEND_ONE; return;
	default: o = (uint32_t)op; s = (uint32_t)sf; d = (uint32_t)df; return;
	}
}

void stencil_face(const VkStencilOpState &v, swgb_stencil_op_state &o)
{
	o.fail_op = (uint32_t)v.failOp;
	o.pass_op = (uint32_t)v.passOp;
	o.depth_fail_op = (uint32_t)v.depthFailOp;
	o.compare_op = (uint32_t)v.compareOp;
	o.compare_mask = v.compareMask;
	o.write_mask = v.writeMask;
	o.reference = v.reference;
	o.reserved = 0;
}

}  // namespace

// Fills *out for a draw of the combined graphics state gs into att, with
// vertex streams inputs, push constants push (the MVP) and, for
// SWGB_FS_TEX_X_VCOLOR, the combined image sampler tex (device finds its
// sampler state).  fs is the fixed fragment shader the pipeline's shader
// matches (the caller recognises it; the bridge does not read SPIR-V).
// Returns false when the draw needs the reference's own path (lines,
// points, non-FILL polygon modes, rasterizer discard, several colour
// attachments or unsupported formats); libswgb rejects, with
// SWGB_UNSUPPORTED_STATE, anything else it does not implement.
bool fill_state(const vk::Device *device, const vk::GraphicsState &gs, const vk::Attachments &att, const vk::Inputs &inputs,
                const vk::Pipeline::PushConstantStorage &push, const vk::SampledImageDescriptor *tex, uint32_t fs, int layer,
                swgb_pipeline_state &out)
{
	std::memset(&out, 0, sizeof(out));
	const vk::VertexInputInterfaceState &vi = gs.getVertexInputInterfaceState();
	const vk::PreRasterizationState &pr = gs.getPreRasterizationState();
	const vk::FragmentState &fr = gs.getFragmentState();
	const vk::FragmentOutputInterfaceState &fo = gs.getFragmentOutputInterfaceState();

	const VkPrimitiveTopology topo = vi.getTopology();
	if(topo != VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST && topo != VK_PRIMITIVE_TOPOLOGY_TRIANGLE_STRIP &&
	   topo != VK_PRIMITIVE_TOPOLOGY_TRIANGLE_FAN)
		return false;
	if(pr.getPolygonMode() != VK_POLYGON_MODE_FILL || pr.hasRasterizerDiscard()) return false;
	if(!att.colorBuffer[0]) return false;
	for(int i = 1; i < sw::MAX_COLOR_BUFFERS; i++)
		if(att.colorBuffer[i]) return false;
	const VkFormat cfmt = att.colorFormat(0);
	if(!supported_color(cfmt)) return false;

	out.topology = (uint32_t)topo;
	out.provoking_vertex = pr.getProvokingVertexMode() == VK_PROVOKING_VERTEX_MODE_LAST_VERTEX_EXT ? 1u : 0u;
	out.precision_profile = SWIFTSHADER_LEGACY_PRECISION ? SWGB_PRECISION_LEGACY : SWGB_PRECISION_CMAKE;

	// vertex streams: attribute k = location k of the fixed vertex shader
	// (position, colour, uv), each from its own stream
	out.attrib_count = 0;
	for(uint32_t i = 0; i < SWGB_MAX_ATTRIBS; i++)
	{
		const sw::Stream &st = inputs.getStream(i);
		if(st.format == VK_FORMAT_UNDEFINED || !st.buffer) break;
		if(st.inputRate != VK_VERTEX_INPUT_RATE_VERTEX) return false;
		out.attribs[i].format = (uint32_t)st.format;
		out.attribs[i].binding = i;
		out.attribs[i].offset = 0;  // sw::Stream::buffer already points at the attribute of vertex 0
		out.bindings[i].buffer = st.buffer;
		out.bindings[i].stride = st.vertexStride;
		out.attrib_count = i + 1;
	}
	out.vertex_shader = SWGB_VS_MVP_PASSTHROUGH;
	out.fragment_shader = fs;
	static_assert(sizeof(push) >= 16 * sizeof(float), "the MVP push-constant block");
	std::memcpy(out.mvp, &push, 16 * sizeof(float));

	// pre-rasterization state (the dynamic state already combined in gs)
	const VkViewport &vp = pr.getViewport();
	out.viewport_x = vp.x;
	out.viewport_y = vp.y;
	out.viewport_width = vp.width;
	out.viewport_height = vp.height;
	out.viewport_min_depth = vp.minDepth;
	out.viewport_max_depth = vp.maxDepth;
	const VkRect2D &sc = pr.getScissor();
	out.scissor_x = sc.offset.x;
	out.scissor_y = sc.offset.y;
	out.scissor_width = sc.extent.width;
	out.scissor_height = sc.extent.height;
	out.cull_mode = (uint32_t)pr.getCullMode();
	out.front_face = (uint32_t)pr.getFrontFace();
	out.depth_clip_enable = pr.getDepthClipEnable() ? 1u : 0u;
	out.depth_clamp_enable = pr.getDepthClampEnable() ? 1u : 0u;
	out.depth_bias_constant = pr.getConstantDepthBias();
	out.depth_bias_slope = pr.getSlopeDepthBias();
	out.depth_bias_clamp = pr.getDepthBiasClamp();

	// colour attachment and blending (location 0)
	const vk::ImageView *color = att.colorBuffer[0];
	const VkExtent2D ext = color->getMipLevelExtent(0);
	out.framebuffer_width = ext.width;
	out.framebuffer_height = ext.height;
	out.color_format = (uint32_t)cfmt;
	out.color = color->getOffsetPointer({ 0, 0, 0 }, VK_IMAGE_ASPECT_COLOR_BIT, 0, layer);
	out.color_pitch_bytes = color->rowPitchBytes(VK_IMAGE_ASPECT_COLOR_BIT, 0);
	out.color_slice_bytes = color->slicePitchBytes(VK_IMAGE_ASPECT_COLOR_BIT, 0);  // sample planes (Renderer.cpp:446-455)
	out.sample_count = (uint32_t)fo.getSampleCount();
	out.color_write_mask = (uint32_t)fo.colorWriteActive(0, att);
	const vk::BlendState b = fo.getBlendState(0, att, false);
	out.blend_enable = b.alphaBlendEnable ? 1u : 0u;
	blend_triple(b.blendOperation, b.sourceBlendFactor, b.destBlendFactor, out.color_blend_op, out.src_color_factor,
	             out.dst_color_factor);
	blend_triple(b.blendOperationAlpha, b.sourceBlendFactorAlpha, b.destBlendFactorAlpha, out.alpha_blend_op,
	             out.src_alpha_factor, out.dst_alpha_factor);

	// depth / stencil
	if(att.depthBuffer)
	{
		out.depth_format = (uint32_t)att.depthFormat();
		out.depth = att.depthBuffer->getOffsetPointer({ 0, 0, 0 }, VK_IMAGE_ASPECT_DEPTH_BIT, 0, layer);
		out.depth_pitch_bytes = att.depthBuffer->rowPitchBytes(VK_IMAGE_ASPECT_DEPTH_BIT, 0);
		out.depth_slice_bytes = att.depthBuffer->slicePitchBytes(VK_IMAGE_ASPECT_DEPTH_BIT, 0);
	}
	out.depth_test_enable = fr.depthTestActive(att) ? 1u : 0u;
	out.depth_write_enable = fr.depthWriteActive(att) ? 1u : 0u;
	out.depth_compare_op = (uint32_t)fr.getDepthCompareMode();
	out.depth_bounds_test_enable = fr.depthBoundsTestActive(att) ? 1u : 0u;
	out.min_depth_bounds = fr.getMinDepthBounds();
	out.max_depth_bounds = fr.getMaxDepthBounds();
	if(att.stencilBuffer && fr.stencilActive(att))
	{
		out.stencil_test_enable = 1;
		out.stencil = att.stencilBuffer->getOffsetPointer({ 0, 0, 0 }, VK_IMAGE_ASPECT_STENCIL_BIT, 0, layer);
		out.stencil_pitch_bytes = att.stencilBuffer->rowPitchBytes(VK_IMAGE_ASPECT_STENCIL_BIT, 0);
		out.stencil_slice_bytes = att.stencilBuffer->slicePitchBytes(VK_IMAGE_ASPECT_STENCIL_BIT, 0);
		stencil_face(fr.getFrontStencil(), out.front);
		stencil_face(fr.getBackStencil(), out.back);
	}

	// the fragment shader's combined image sampler: the descriptor's sw::Texture
	// (WriteTextureLevelInfo, VkDescriptorSetLayout.cpp:299-331) and its sampler
	if(fs == SWGB_FS_TEX_X_VCOLOR)
	{
		if(!tex || !device) return false;
		const vk::SamplerState *ss = device->findSampler(tex->samplerId);
		if(!ss) return false;
		swgb_texture &t = out.texture;
		t.format = (uint32_t)tex->memoryOwner->getFormat();
		const int levels = tex->mipLevels < SWGB_MAX_MIP_LEVELS ? tex->mipLevels : SWGB_MAX_MIP_LEVELS;
		t.level_count = (uint32_t)levels;
		for(int l = 0; l < levels; l++)
		{
			const sw::Mipmap &m = tex->texture.mipmap[l];
			t.levels[l].buffer = m.buffer;
			t.levels[l].width = m.width[0];
			t.levels[l].height = m.height[0];
			t.levels[l].pitch_texels = m.pitchP[0];
		}
		t.mag_filter = (uint32_t)ss->magFilter;
		t.min_filter = (uint32_t)ss->minFilter;
		t.mipmap_mode = (uint32_t)ss->mipmapMode;
		t.address_u = (uint32_t)ss->addressModeU;
		t.address_v = (uint32_t)ss->addressModeV;
		t.mip_lod_bias = ss->mipLodBias;
		t.min_lod = ss->minLod;
		t.max_lod = ss->maxLod;
		t.border_color = (uint32_t)ss->borderColor;
		for(int c = 0; c < 4; c++) t.custom_border_color[c] = ss->customBorderColor.float32[c];
	}
	return true;
}

// The arguments of sw::Renderer::draw (src/Device/Renderer.hpp:211-213) as
// swgb_draw_args: count is the primitive count Renderer::draw receives;
// vertexCount bounds every index + baseVertex (libswgb transforms each vertex
// once instead of through the vertex cache); restartIndexCount is nonzero to
// let libswgb split a primitive-restart index range itself (instead of
// vk::IndexBuffer::getIndexBuffers, src/Device/Context.cpp:49-91).
void fill_args(unsigned int count, int baseVertex, uint32_t firstVertex, const void *indexBuffer, VkIndexType indexType,
               uint32_t vertexCount, int instanceID, int layer, const VkRect2D &renderArea, uint32_t restartIndexCount,
               swgb_draw_args &out)
{
	std::memset(&out, 0, sizeof(out));
	out.count = count;
	out.base_vertex = baseVertex;
	out.first_vertex = firstVertex;
	out.index_type = indexBuffer ? (uint32_t)indexType : SWGB_INDEX_TYPE_NONE;
	out.indices = indexBuffer;
	out.vertex_count = vertexCount;
	out.instance_id = instanceID;
	out.layer = layer;
	out.render_area_x = renderArea.offset.x;
	out.render_area_y = renderArea.offset.y;
	out.render_area_width = renderArea.extent.width;
	out.render_area_height = renderArea.extent.height;
	out.restart_index_count = restartIndexCount;
	// the queue has already ordered every texture write before the draw
	out.raster_wait_event = nullptr;
}

}  // namespace swgb_bridge
