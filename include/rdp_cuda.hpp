/*
 * Header-only C++ face of librdp_cuda (rdp_cuda.h) in the shape of the reference's
 * RDP::CommandProcessor (parallel-rdp/rdp_device.hpp:111-197), so that an emulator written against
 * that class switches by changing its include and its device argument:
 *
 *   reference:  RDP::CommandProcessor cp(vulkan_device, rdram, 0, rdram_size, rdram_size / 2, flags);
 *   this:       RDP::CommandProcessor cp(cuda_device_ordinal, rdram, 0, rdram_size, rdram_size / 2, flags);
 *
 * Same method names, argument meanings and error behaviour: no exceptions; an unusable device or an
 * unsupported configuration makes device_is_supported() return false and the other methods do
 * nothing.  Differences follow from the device API: scanout() returns the image in device memory
 * (ScanoutImage) instead of a Vulkan image and scanout_async_buffer() fills a VIScanoutBuffer whose
 * fence is a CUDA event.  Upscaling and super-sampled readback follow the reference's flags (an
 * upscaling processor needs hidden_rdram_size == rdram_size / 2).
 */
#ifndef RDP_CUDA_HPP
#define RDP_CUDA_HPP

#include <stdint.h>
#include <string.h>
#include <vector>

#include "rdp_cuda.h"

namespace RDP
{
struct RGBA
{
	uint8_t r, g, b, a;
};

// rdp_device.hpp:43-53.
enum CommandProcessorFlagBits
{
	COMMAND_PROCESSOR_FLAG_HOST_VISIBLE_HIDDEN_RDRAM_BIT = 1 << 0,
	COMMAND_PROCESSOR_FLAG_HOST_VISIBLE_TMEM_BIT = 1 << 1,
	COMMAND_PROCESSOR_FLAG_UPSCALING_2X_BIT = 1 << 2,
	COMMAND_PROCESSOR_FLAG_UPSCALING_4X_BIT = 1 << 3,
	COMMAND_PROCESSOR_FLAG_UPSCALING_8X_BIT = 1 << 4,
	COMMAND_PROCESSOR_FLAG_SUPER_SAMPLED_READ_BACK_BIT = 1 << 5,
	COMMAND_PROCESSOR_FLAG_SUPER_SAMPLED_DITHER_BIT = 1 << 6,
	// Decode commands on a thread of the processor (the reference's default; it decodes on the
	// caller's thread under PARALLEL_RDP_SINGLE_THREADED_COMMAND, which is this library's default).
	COMMAND_PROCESSOR_FLAG_COMMAND_THREAD_BIT = 1 << 16
};
using CommandProcessorFlags = uint32_t;

// rdp_device.hpp:77-109: the options travel in band as one word (MetaSetQuirks).
struct Quirks
{
	Quirks()
	{
		u.words[0] = 0;
		u.options.native_resolution_tex_rect = true;
		u.options.native_texture_lod = false;
	}
	void set_native_resolution_tex_rect(bool enable) { u.options.native_resolution_tex_rect = enable; }
	void set_native_texture_lod(bool enable) { u.options.native_texture_lod = enable; }
	union
	{
		struct Opts
		{
			bool native_resolution_tex_rect;
			bool native_texture_lod;
		} options;
		uint32_t words[1];
	} u;
};

// rdp_common.hpp: VI register indices.
enum class VIRegister
{
	Control = 0, Origin, Width, Intr, VCurrentLine, Timing, VSync, HSync, Leap, HStart, VStart, VBurst, XScale, YScale,
	Count
};

// rdp_renderer.hpp:75-95.
enum class ValidationError
{
	Fill4bpp,
	LoadTile4bpp,
	InvalidMultilineLoadTlut,
	FillDepthTest,
	FillDepthWrite,
	FillImageReadEnable,
	Copy32bpp
};

class ValidationInterface
{
public:
	virtual ~ValidationInterface() = default;
	virtual void report_rdp_crash(ValidationError err, const char *msg) = 0;
};

// video_interface.hpp:31-81 (the export fields have no counterpart: there is no graphics API here).
struct ScanoutOptions
{
	unsigned crop_overscan_pixels = 0;
	struct CropRect
	{
		unsigned left = 0;
		unsigned right = 0;
		unsigned top = 0;
		unsigned bottom = 0;
		bool enable = false;
	} crop_rect;
	unsigned downscale_steps = 0;
	bool persist_frame_on_invalid_input = false;
	bool blend_previous_frame = false;
	bool upscale_deinterlacing = true;
	struct
	{
		bool aa = true;
		bool scale = true;
		bool serrate = true;
		bool dither_filter = true;
		bool divot_filter = true;
		bool gamma_dither = true;
	} vi;
};

// The scanout image in device memory (the reference returns a Vulkan image handle).
struct ScanoutImage
{
	const uint32_t *pixels = nullptr; // device pointer, RGBA8; null: no image
	unsigned width = 0, height = 0;
	explicit operator bool() const { return pixels != nullptr; }
};

// video_interface.hpp:83-89.
struct VIScanoutBuffer
{
	rdp_vi_scanout_buffer buf = {};
	unsigned width = 0, height = 0;
	struct Fence
	{
		rdp_vi_scanout_buffer *b = nullptr;
		void wait() { if (b) rdp_vi_scanout_buffer_wait(b, UINT64_MAX); }
	} fence;
	const uint32_t *data() const { return buf.pixels; }
	VIScanoutBuffer() = default;
	VIScanoutBuffer(const VIScanoutBuffer &) = delete;
	VIScanoutBuffer &operator=(const VIScanoutBuffer &) = delete;
	~VIScanoutBuffer() { rdp_vi_scanout_buffer_release(&buf); }
};

namespace VideoInterface
{
enum PerScanlineRegisterBits
{
	PER_SCANLINE_HSTART_BIT = 1 << 0,
	PER_SCANLINE_XSCALE_BIT = 1 << 1
};
using PerScanlineRegisterFlags = uint32_t;
} // namespace VideoInterface

class CommandProcessor
{
public:
	CommandProcessor(int device, void *rdram_ptr, size_t rdram_offset, size_t rdram_size, size_t hidden_rdram_size,
	                 CommandProcessorFlags flags)
	{
		rdp_create_info info = {};
		info.rdram = rdram_ptr;
		info.rdram_offset = rdram_offset;
		info.rdram_size = rdram_size;
		info.hidden_rdram_size = hidden_rdram_size;
		info.flags = (flags & COMMAND_PROCESSOR_FLAG_COMMAND_THREAD_BIT) ? RDP_CREATE_COMMAND_THREAD : 0u;
		if (flags & COMMAND_PROCESSOR_FLAG_UPSCALING_2X_BIT) info.flags |= RDP_CREATE_UPSCALING_2X;
		if (flags & COMMAND_PROCESSOR_FLAG_UPSCALING_4X_BIT) info.flags |= RDP_CREATE_UPSCALING_4X;
		if (flags & COMMAND_PROCESSOR_FLAG_UPSCALING_8X_BIT) info.flags |= RDP_CREATE_UPSCALING_8X;
		if (flags & COMMAND_PROCESSOR_FLAG_SUPER_SAMPLED_READ_BACK_BIT) info.flags |= RDP_CREATE_SUPER_SAMPLED_READ_BACK;
		if (flags & COMMAND_PROCESSOR_FLAG_SUPER_SAMPLED_DITHER_BIT) info.flags |= RDP_CREATE_SUPER_SAMPLED_DITHER;
		info.device = device;
		if (rdp_cp_create(&info, &cp) != RDP_OK) cp = nullptr;
	}
	~CommandProcessor() { rdp_cp_destroy(cp); }
	CommandProcessor(const CommandProcessor &) = delete;
	CommandProcessor &operator=(const CommandProcessor &) = delete;

	void set_validation_interface(ValidationInterface *iface)
	{
		validation = iface;
		if (cp) rdp_cp_set_validation_callback(cp, iface ? &CommandProcessor::on_validation : nullptr, this);
	}

	bool device_is_supported() const { return cp != nullptr; }

	// Synchronization.
	void flush() { if (cp) rdp_cp_flush(cp); }
	uint64_t signal_timeline()
	{
		uint64_t v = 0;
		if (cp) rdp_cp_signal_timeline(cp, &v);
		return v;
	}
	void wait_for_timeline(uint64_t index) { if (cp) rdp_cp_wait_timeline(cp, index, UINT64_MAX); }
	void idle() { if (cp) rdp_cp_idle(cp); }
	void begin_frame_context() { if (cp) rdp_cp_begin_frame_context(cp); }

	// Queues up state and drawing commands.
	void enqueue_command(unsigned num_words, const uint32_t *words) { if (cp) rdp_cp_enqueue(cp, num_words, words); }
	void enqueue_command_direct(unsigned num_words, const uint32_t *words) { enqueue_command(num_words, words); }

	void set_quirks(const Quirks &quirks) { if (cp) rdp_cp_set_quirks(cp, quirks.u.words[0]); }

	// Interact with memory.
	void *begin_read_rdram() { return cp ? rdp_cp_begin_read_rdram(cp) : nullptr; }
	void end_write_rdram() { if (cp) rdp_cp_end_write_rdram(cp); }
	void *begin_read_hidden_rdram() { return cp ? rdp_cp_begin_read_hidden_rdram(cp) : nullptr; }
	void end_write_hidden_rdram() { if (cp) rdp_cp_end_write_hidden_rdram(cp); }
	size_t get_rdram_size() const { return cp ? rdp_cp_get_rdram_size(cp) : 0; }
	size_t get_hidden_rdram_size() const { return cp ? rdp_cp_get_hidden_rdram_size(cp) : 0; }
	// The internal upscaling factor (Renderer::get_scaling_factor, rdp_renderer.cpp:2694-2697).
	unsigned get_scaling_factor() const { return cp ? rdp_cp_get_scaling_factor(cp) : 1u; }
	// TMEM as 2048 16-bit words (a host copy, current when the call returns).
	void *get_tmem()
	{
		if (!cp || rdp_cp_get_tmem(cp, tmem_copy) != RDP_OK) return nullptr;
		return tmem_copy;
	}

	void set_vi_register(VIRegister reg, uint32_t value) { if (cp) rdp_cp_set_vi_register(cp, uint32_t(reg), value); }

	ScanoutImage scanout(const ScanoutOptions &opts = {})
	{
		ScanoutImage img;
		rdp_vi_image out = {};
		rdp_scanout_options o = convert(opts);
		if (cp && rdp_cp_scanout(cp, &o, &out) == RDP_OK && out.pixels)
		{
			img.pixels = out.pixels;
			img.width = out.width;
			img.height = out.height;
		}
		return img;
	}
	void scanout_sync(std::vector<RGBA> &colors, unsigned &width, unsigned &height, const ScanoutOptions &opts = {})
	{
		VIScanoutBuffer scanout;
		scanout_async_buffer(scanout, opts);
		width = scanout.width;
		height = scanout.height;
		if (!width || !height)
		{
			colors.clear();
			return;
		}
		colors.resize(size_t(width) * height);
		scanout.fence.wait();
		memcpy(colors.data(), scanout.data(), size_t(width) * height * sizeof(uint32_t));
	}
	void scanout_async_buffer(VIScanoutBuffer &buffer, const ScanoutOptions &opts = {})
	{
		rdp_scanout_options o = convert(opts);
		buffer.width = buffer.height = 0;
		buffer.fence.b = nullptr;
		if (!cp || rdp_cp_scanout_async_buffer(cp, &o, &buffer.buf) != RDP_OK) return;
		buffer.width = buffer.buf.width;
		buffer.height = buffer.buf.height;
		if (buffer.width) buffer.fence.b = &buffer.buf;
	}

	// Per-scanline VI registers (rdp_device.hpp:154-197).
	void begin_vi_register_per_scanline(VideoInterface::PerScanlineRegisterFlags flags)
	{
		if (cp) rdp_cp_begin_vi_register_per_scanline(cp, flags);
	}
	void set_vi_register_for_scanline(VideoInterface::PerScanlineRegisterBits reg, uint32_t value)
	{
		if (cp) rdp_cp_set_vi_register_for_scanline(cp, uint32_t(reg), value);
	}
	void latch_vi_register_for_scanline(unsigned vi_line) { if (cp) rdp_cp_latch_vi_register_for_scanline(cp, vi_line); }
	void end_vi_register_per_scanline() { if (cp) rdp_cp_end_vi_register_per_scanline(cp); }

	// The underlying C handle (for the library's extensions: batches, capture, statistics).
	rdp_cp *handle() const { return cp; }

private:
	rdp_cp *cp = nullptr;
	ValidationInterface *validation = nullptr;
	uint16_t tmem_copy[2048] = {};

	static rdp_scanout_options convert(const ScanoutOptions &s)
	{
		rdp_scanout_options o;
		rdp_scanout_options_default(&o);
		o.crop_overscan_pixels = s.crop_overscan_pixels;
		o.crop_rect_enable = s.crop_rect.enable;
		o.crop_left = s.crop_rect.left;
		o.crop_right = s.crop_rect.right;
		o.crop_top = s.crop_rect.top;
		o.crop_bottom = s.crop_rect.bottom;
		o.persist_frame_on_invalid_input = s.persist_frame_on_invalid_input;
		o.blend_previous_frame = s.blend_previous_frame;
		o.upscale_deinterlacing = s.upscale_deinterlacing;
		o.vi_aa = s.vi.aa;
		o.vi_scale = s.vi.scale;
		o.vi_serrate = s.vi.serrate;
		o.vi_dither_filter = s.vi.dither_filter;
		o.vi_divot_filter = s.vi.divot_filter;
		o.vi_gamma_dither = s.vi.gamma_dither;
		o.downscale_steps = s.downscale_steps < 8 ? s.downscale_steps : 8; // video_interface.cpp:1217
		return o;
	}

	static void on_validation(void *user, int error, const char *message)
	{
		auto *self = static_cast<CommandProcessor *>(user);
		if (!self->validation) return;
		ValidationError e = ValidationError::Fill4bpp;
		switch (error)
		{
		case RDP_VALIDATION_FILL_4BPP: e = ValidationError::Fill4bpp; break;
		case RDP_VALIDATION_FILL_DEPTH_TEST: e = ValidationError::FillDepthTest; break;
		case RDP_VALIDATION_FILL_DEPTH_WRITE: e = ValidationError::FillDepthWrite; break;
		case RDP_VALIDATION_FILL_IMAGE_READ: e = ValidationError::FillImageReadEnable; break;
		case RDP_VALIDATION_COPY_32BPP: e = ValidationError::Copy32bpp; break;
		case RDP_VALIDATION_LOAD_TILE_4BPP: e = ValidationError::LoadTile4bpp; break;
		case RDP_VALIDATION_MULTILINE_TLUT: e = ValidationError::InvalidMultilineLoadTlut; break;
		default: return;
		}
		self->validation->report_rdp_crash(e, message);
	}
};
} // namespace RDP

#endif
