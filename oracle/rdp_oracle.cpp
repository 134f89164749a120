/*
 * CPU ORACLE for the N64 RDP rendering path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py.  It is never linked into, called by or loaded
 * by the product library (parallel-rdp_gb300/csrc).
 *
 * It restates, in plain scalar C++, the fixed-point arithmetic of the
 * reference (Themaister/parallel-rdp) for the RDP path:
 *   - command decode:        parallel-rdp/rdp_device.cpp:268-864
 *   - primitive set-up:      parallel-rdp/rdp_renderer.cpp:717-1562
 *   - TMEM upload planning:  parallel-rdp/rdp_renderer.cpp:3099-3486
 *   - TMEM update:           parallel-rdp/shaders/tmem_update.comp
 *   - span set-up:           parallel-rdp/shaders/span_setup.comp
 *   - conservative binning:  parallel-rdp/shaders/binning.h
 *   - per-pixel shading:     parallel-rdp/shaders/shading.h (+ coverage.h,
 *     interpolation.h, clamping.h, perspective.h, texture.h, combiner.h,
 *     dither.h, noise.h)
 *   - depth / blend / RDRAM: parallel-rdp/shaders/memory_interfacing.h,
 *     depth_test.h, blender.h, z_encode.h, depth_blend.comp, ubershader.comp
 *
 * Unlike the reference (which batches <=256 primitives into render passes and
 * bins them into 8x8 tiles on the GPU), the oracle renders every primitive
 * immediately, pixel by pixel, in stream order.  The pass structure only
 * affects results through the global primitive index used to seed noise
 * (rdp_renderer.cpp:2346, 2913) and the TMEM state a primitive samples
 * (tmem_update.comp:546-576); the oracle reproduces both by construction:
 * noise is seeded with the running primitive count and TMEM loads are applied
 * in stream order.
 *
 * Parity of this restatement against Angrylion-Plus (the reference's own
 * oracle) is unpinned: that dependency is an empty submodule in the reference
 * tree and cannot be built.  See tests/test_oracle_known_answers.py for the
 * hand-derived known-answer checks that pin its fixed-point primitives.
 *
 * Build: g++ -O2 -fwrapv -std=c++20 -shared -fPIC (see oracle/Makefile).
 */
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#include <vector>
#include <algorithm>
#include <memory>

#include "../parallel-rdp_gb300/csrc/blender_divider_runs.inc"

namespace {

// ----------------------------------------------------------------------------
// GLSL helpers.
static inline int bfe_s(int v, int bits) { return int(uint32_t(v) << (32 - bits)) >> (32 - bits); }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline int find_lsb(uint32_t v) { return v ? __builtin_ctz(v) : -1; }
static inline int find_msb(int v)
{
	if (v < 0) v = ~v;
	return v ? 31 - __builtin_clz(uint32_t(v)) : -1;
}
static inline int popc(uint32_t v) { return __builtin_popcount(v); }

// ----------------------------------------------------------------------------
// Flag constants (parallel-rdp/rdp_data_structures.hpp:31-93).
enum
{
	TRI_FLIP = 1 << 0, TRI_DO_OFFSET = 1 << 1, TRI_SKIP_XFRAC = 1 << 2, TRI_INTERLACE_FIELD = 1 << 3,
	TRI_INTERLACE_KEEP_ODD = 1 << 4, TRI_DISABLE_UPSCALING = 1 << 5, TRI_NATIVE_LOD = 1 << 6,
	TRI_FILL_COPY_RASTER = 1 << 7
};

enum : uint32_t
{
	R_INTERLACE_FIELD = 1u << 0, R_INTERLACE_KEEP_ODD = 1u << 1, R_AA = 1u << 2, R_PERSPECTIVE = 1u << 3,
	R_TLUT = 1u << 4, R_TLUT_TYPE = 1u << 5, R_CVG_TIMES_ALPHA = 1u << 6, R_ALPHA_CVG_SELECT = 1u << 7,
	R_MULTI_CYCLE = 1u << 8, R_TEX_LOD = 1u << 9, R_SHARPEN = 1u << 10, R_DETAIL = 1u << 11,
	R_FILL = 1u << 12, R_COPY = 1u << 13, R_SAMPLE_QUAD = 1u << 14, R_ALPHA_TEST = 1u << 15,
	R_ALPHA_TEST_DITHER = 1u << 16, R_MID_TEXEL = 1u << 17, R_USES_TEXEL0 = 1u << 18,
	R_USES_TEXEL1 = 1u << 19, R_USES_LOD = 1u << 20, R_USES_PIPELINED_TEXEL1 = 1u << 21,
	R_CONVERT_ONE = 1u << 22, R_BILERP0 = 1u << 23, R_BILERP1 = 1u << 24, R_NEED_NOISE_DUAL = 1u << 25,
	R_NEED_NOISE = 1u << 28, R_STATIC_TEX = 1u << 29
};

enum : uint32_t
{
	DB_DEPTH_TEST = 1u << 0, DB_DEPTH_UPDATE = 1u << 1, DB_FORCE_BLEND = 1u << 3, DB_IMAGE_READ = 1u << 4,
	DB_COLOR_ON_CVG = 1u << 5, DB_MULTI_CYCLE = 1u << 6, DB_AA = 1u << 7, DB_DITHER = 1u << 8
};

enum { TILE_CLAMP_S = 1, TILE_MIRROR_S = 2, TILE_CLAMP_T = 4, TILE_MIRROR_T = 8 };
enum { FB_I4 = 0, FB_I8 = 1, FB_RGBA5551 = 2, FB_IA88 = 3, FB_RGBA8888 = 4 };
enum { FMT_RGBA = 0, FMT_YUV = 1, FMT_CI = 2, FMT_IA = 3, FMT_I = 4 };
enum { MODE_TILE = 0, MODE_TLUT = 1, MODE_BLOCK = 2 };

struct TriSetup
{
	int xh, xm, xl;
	int yh, ym;
	int dxhdy, dxmdy, dxldy;
	int yl;
	uint32_t flags;
	uint32_t tile;
};

struct Attr
{
	int rgba[4], drgba_dx[4], drgba_de[4], drgba_dy[4];
	int stzw[4], dstzw_dx[4], dstzw_de[4], dstzw_dy[4]; // s, t, z, w
};

struct TileInfo
{
	uint32_t slo, shi, tlo, thi;
	uint32_t offset, stride;
	int fmt, size, palette, mask_s, shift_s, mask_t, shift_t, flags;
};

struct StaticState
{
	int rgb[2][4];   // muladd, mulsub, mul, add
	int alpha[2][4]; // muladd, mulsub, mul, add
	uint32_t flags;
	int dither;
};

struct BlendModes { int m1a, m1b, m2a, m2b; };

struct DepthBlend
{
	BlendModes cyc[2];
	uint32_t flags;
	int coverage_mode;
	int z_mode;
};

struct Derived
{
	int c_muladd[2][4], c_mulsub[2][4], c_mul[2][4], c_add[2][4];
	int fog[4], blend[4];
	uint32_t fill_color;
	int dz, dz_compressed, min_lod;
	int factors[4];
};

struct Scissor { int xlo, ylo, xhi, yhi; };

struct Span
{
	int rgba[4];
	int stzw[4];
	int xleft[4], xright[4];
	int base_x, start_x, end_x, lodlength;
	bool valid;
};

struct PixelStateSlot
{
	int color[4];
	bool color_dirty;
	int depth;
	int dz;
	bool depth_dirty;
	uint32_t color_index;
	uint32_t pass_stamp;
};

struct UploadInfo
{
	int width, height;
	float min_t_mod, max_t_mod;
	int vram_addr, vram_width, vram_size, vram_effective_width;
	int tmem_offset, tmem_stride_words, tmem_size, tmem_fmt;
	int mode;
	float inv_tmem_stride_words;
	int dxt;
};

// Dither matrices (parallel-rdp/shaders/dither.h:28-30): magic square and Bayer.
static const uint8_t dither_matrices[2][16] = {
	{ 0, 6, 1, 7, 4, 2, 5, 3, 3, 5, 2, 4, 7, 1, 6, 0 },
	{ 0, 4, 1, 5, 4, 0, 5, 1, 3, 7, 2, 6, 7, 3, 6, 2 },
};

// Reciprocal table for the perspective divider (parallel-rdp/shaders/perspective.h:27-44):
// {base, slope} with slope pre-multiplied by 4.
static const int16_t persp_base[64] = {
	0x4000, 0x3f04, 0x3e10, 0x3d22, 0x3c3c, 0x3b5d, 0x3a83, 0x39b1, 0x38e4, 0x381c, 0x375a, 0x369d, 0x35e5, 0x3532, 0x3483, 0x33d9,
	0x3333, 0x3291, 0x31f4, 0x3159, 0x30c3, 0x3030, 0x2fa1, 0x2f15, 0x2e8c, 0x2e06, 0x2d83, 0x2d03, 0x2c86, 0x2c0b, 0x2b93, 0x2b1e,
	0x2aab, 0x2a3a, 0x29cc, 0x2960, 0x28f6, 0x288e, 0x2828, 0x27c4, 0x2762, 0x2702, 0x26a4, 0x2648, 0x25ed, 0x2594, 0x253d, 0x24e7,
	0x2492, 0x243f, 0x23ee, 0x239e, 0x234f, 0x2302, 0x22b6, 0x226c, 0x2222, 0x21da, 0x2193, 0x214d, 0x2108, 0x20c5, 0x2082, 0x2041,
};
static const int16_t persp_slope[64] = {
	252, 244, 238, 230, 223, 218, 210, 205, 200, 194, 189, 184, 179, 175, 170, 166,
	162, 157, 155, 150, 147, 143, 140, 137, 134, 131, 128, 125, 123, 120, 117, 115,
	113, 110, 108, 106, 104, 102, 100, 98, 96, 94, 92, 91, 89, 87, 86, 85,
	83, 81, 80, 79, 77, 76, 74, 74, 72, 71, 70, 69, 67, 67, 65, 65,
};

// ----------------------------------------------------------------------------
// The oracle processor state.
struct Oracle
{
	// Reference render-pass count (the unit of the throughput metric): the reference ends a
	// pass on need_flush (rdp_renderer.cpp:1564-1590: 256 primitives, 64 distinct static
	// states, 64 distinct depth-blend states, span-job budget), before the 256th TMEM
	// upload (3484-3485) and on every hard flush (image changes, SyncFull, load hazards).
	struct RefPasses
	{
		uint64_t passes = 0;
		uint32_t prims = 0, uploads = 0, span_jobs = 0;
		std::vector<uint64_t> static_keys, depth_keys;
		void cut()
		{
			passes++;
			prims = uploads = span_jobs = 0;
			static_keys.clear();
			depth_keys.clear();
		}
		void hard() { if (prims || uploads) cut(); }
		void upload() { if (++uploads + 1 >= 256) cut(); }
		void prim(uint32_t om0, uint32_t om1, uint32_t c0, uint32_t c1, int lines)
		{
			uint64_t skey = (uint64_t(om0) << 32) ^ (uint64_t(om1 & 0x3f0fu) << 20) ^ uint64_t(c0) ^ (uint64_t(c1) << 7);
			uint64_t dkey = (uint64_t(om1) << 8) | ((om0 >> 20) & 3);
			if (std::find(static_keys.begin(), static_keys.end(), skey) == static_keys.end()) static_keys.push_back(skey);
			if (std::find(depth_keys.begin(), depth_keys.end(), dkey) == depth_keys.end()) depth_keys.push_back(dkey);
			prims++;
			if (lines > 0) span_jobs += uint32_t((lines + 2 + 63) / 64);
			if (prims >= 256 || static_keys.size() >= 64 || depth_keys.size() >= 64 || span_jobs * 64 + 1024 > 32 * 1024)
				cut();
		}
		uint64_t total() const { return passes + ((prims || uploads) ? 1 : 0); }
	} ref;
	uint32_t raw_other_modes[2] = { 0, 0 }, raw_combine[2] = { 0, 0 };

	std::vector<uint8_t> rdram;
	std::vector<uint8_t> hidden;
	uint32_t rdram_size = 0;
	uint32_t hidden_size = 0;
	uint16_t tmem[2048] = {};
	uint8_t blender_lut[0x8000];

	// Command-processor state (rdp_device.hpp).
	StaticState static_state = {};
	DepthBlend depth_blend = {};
	Scissor scissor = {};
	TileInfo tiles[8] = {};
	struct { uint32_t addr = 0, width = 0, size = 0; int fmt = 0; } texture_image;

	// Renderer state.
	struct
	{
		uint32_t addr = 0, depth_addr = 0, width = 0;
		int fmt = FB_RGBA5551;
	} fb;

	struct
	{
		uint32_t blend_color = 0, fog_color = 0, env_color = 0, primitive_color = 0, fill_color = 0;
		int prim_lod_frac = 0, min_level = 0;
		int convert[6] = {};
		int key_width[3] = {}, key_center[3] = {}, key_scale[3] = {};
		int prim_depth = 0, prim_dz = 0;
		bool use_prim_depth = false;
	} constants;

	uint32_t quirks = 1; // native_resolution_tex_rect on by default (rdp_device.hpp:79-83)
	void *vi_state = nullptr; // owned VI oracle state (vi_oracle.cpp)

	// Render-pass model.  The reference keeps a tile's colour/depth in registers for a
	// whole render pass (init_tile/finish_tile, memory_interfacing.h:286-362): pixels are
	// loaded at their first use in a pass and stored when the pass ends.  For I8 colour
	// images and colour/depth aliasing that store/reload round trip is not transparent, so
	// pass boundaries are observable; they follow the reference's segmentation: every 256
	// primitives (Limits::MaxPrimitives), before the 256th TMEM upload, on colour/depth
	// image changes, on TMEM loads that read pending framebuffer writes
	// (rdp_renderer.cpp:3051-3097) and on SyncFull.
	std::vector<PixelStateSlot> pixel_cache;
	std::vector<uint32_t> touched;
	uint32_t pass_prims = 0, pass_uploads = 0, deduced_height = 0;
	bool color_pending = false, depth_pending = false;
	uint32_t pass_span_prims = 0;   // primitives of the pass with span rows (the reference's span jobs)
	uint32_t primitive_counter = 0; // running count == base_primitive_index + index in pass
	uint64_t fragments = 0;         // depth_blend/fill/copy executions

	// Per-pixel noise state (noise.h).
	uint32_t seeded_noise = 0;

	// ------------------------------------------------------------------ RDRAM access
	uint32_t mask8() const { return rdram_size - 1; }
	// The memory the pixel accessors address: RDRAM and hidden RDRAM, or one sample slice of their
	// multisampled copies while a pass renders upscaled.
	uint8_t *mem_rd = nullptr, *mem_hd = nullptr;
	uint8_t vram8(uint32_t i) const { return mem_rd[i & (rdram_size - 1)]; }
	void w_vram8(uint32_t i, uint8_t v) { mem_rd[i & (rdram_size - 1)] = v; }
	uint16_t vram16(uint32_t i) const
	{
		uint32_t b = (i * 2) & (rdram_size - 1);
		return uint16_t(mem_rd[b] | (mem_rd[b + 1] << 8));
	}
	void w_vram16(uint32_t i, uint16_t v)
	{
		uint32_t b = (i * 2) & (rdram_size - 1);
		mem_rd[b] = uint8_t(v);
		mem_rd[b + 1] = uint8_t(v >> 8);
	}
	uint32_t vram32(uint32_t i) const
	{
		uint32_t b = (i * 4) & (rdram_size - 1);
		return uint32_t(mem_rd[b]) | (uint32_t(mem_rd[b + 1]) << 8) | (uint32_t(mem_rd[b + 2]) << 16) |
		       (uint32_t(mem_rd[b + 3]) << 24);
	}
	void w_vram32(uint32_t i, uint32_t v)
	{
		uint32_t b = (i * 4) & (rdram_size - 1);
		mem_rd[b] = uint8_t(v);
		mem_rd[b + 1] = uint8_t(v >> 8);
		mem_rd[b + 2] = uint8_t(v >> 16);
		mem_rd[b + 3] = uint8_t(v >> 24);
	}
	uint8_t hid(uint32_t i) const { return mem_hd[i & (hidden_size - 1)]; }
	void w_hid(uint32_t i, uint8_t v) { mem_hd[i & (hidden_size - 1)] = v; }

	// TMEM byte view of the 16-bit words (tmem8 aliases tmem16 on a little-endian buffer).
	static uint8_t tm8(const uint16_t *t, uint32_t i) { return uint8_t(t[(i >> 1) & 2047] >> ((i & 1) * 8)); }

	void init_luts()
	{
		for (int d = 0; d < 16; d++)
			for (int n = 0; n < 2048; n++)
				blender_lut[(d << 11) | n] = d ? uint8_t((n / d) & 0xff) : 0;
		for (int i = 0; i < RDP_BLENDER_DIVIDER_NUM_RUNS; i++)
		{
			const unsigned short *r = rdp_blender_divider_runs[i];
			for (int k = 0; k < r[2]; k++)
				blender_lut[(r[0] << 11) | (r[1] + k)] = uint8_t(r[3]);
		}
	}

	// ======================================================================= decode
	// rdp_device.cpp:268-294
	void decode_triangle_setup(TriSetup &s, const uint32_t *w) const
	{
		bool copy_cycle = (static_state.flags & R_COPY) != 0;
		bool flip = (w[0] & 0x800000u) != 0;
		bool sign_dxhdy = (w[5] & 0x80000000u) != 0;
		bool do_offset = flip == sign_dxhdy;
		s = {};
		s.flags |= flip ? TRI_FLIP : 0;
		s.flags |= do_offset ? TRI_DO_OFFSET : 0;
		s.flags |= copy_cycle ? TRI_SKIP_XFRAC : 0;
		s.flags |= (quirks & 0xff00u) ? TRI_NATIVE_LOD : 0;
		s.tile = (w[0] >> 16) & 63;
		s.yl = bfe_s(int(w[0]), 14);
		s.ym = bfe_s(int(w[1] >> 16), 14);
		s.yh = bfe_s(int(w[1]), 14);
		s.xl = bfe_s(int(w[2]), 28) >> 1;
		s.xh = bfe_s(int(w[4]), 28) >> 1;
		s.xm = bfe_s(int(w[6]), 28) >> 1;
		s.dxldy = bfe_s(int(w[3] >> 2), 28) >> 1;
		s.dxhdy = bfe_s(int(w[5] >> 2), 28) >> 1;
		s.dxmdy = bfe_s(int(w[7] >> 2), 28) >> 1;
	}

	// rdp_device.cpp:315-336
	static void decode_rgba(Attr &a, const uint32_t *w)
	{
		for (int c = 0; c < 4; c++)
		{
			int wi = c >> 1;
			bool lo = (c & 1) != 0;
			auto merge = [&](int hi_word, int lo_word) -> int {
				uint32_t h = lo ? (w[hi_word] << 16) : (w[hi_word] & 0xffff0000u);
				uint32_t l = lo ? (w[lo_word] & 0xffff) : ((w[lo_word] >> 16) & 0xffff);
				return int(h | l);
			};
			a.rgba[c] = merge(0 + wi, 4 + wi);
			a.drgba_dx[c] = merge(2 + wi, 6 + wi);
			a.drgba_de[c] = merge(8 + wi, 12 + wi);
			a.drgba_dy[c] = merge(10 + wi, 14 + wi);
		}
	}

	// rdp_device.cpp:296-313
	static void decode_tex(Attr &a, const uint32_t *w)
	{
		auto hi = [](uint32_t x) { return x & 0xffff0000u; };
		auto lo16 = [](uint32_t x) { return (x >> 16) & 0xffffu; };
		a.stzw[0] = int(hi(w[0]) | lo16(w[4]));
		a.stzw[1] = int(((w[0] << 16) & 0xffff0000u) | (w[4] & 0xffffu));
		a.stzw[3] = int(hi(w[1]) | lo16(w[5]));
		a.dstzw_dx[0] = int(hi(w[2]) | lo16(w[6]));
		a.dstzw_dx[1] = int(((w[2] << 16) & 0xffff0000u) | (w[6] & 0xffffu));
		a.dstzw_dx[3] = int(hi(w[3]) | lo16(w[7]));
		a.dstzw_de[0] = int(hi(w[8]) | lo16(w[12]));
		a.dstzw_de[1] = int(((w[8] << 16) & 0xffff0000u) | (w[12] & 0xffffu));
		a.dstzw_de[3] = int(hi(w[9]) | lo16(w[13]));
		a.dstzw_dy[0] = int(hi(w[10]) | lo16(w[14]));
		a.dstzw_dy[1] = int(((w[10] << 16) & 0xffff0000u) | (w[14] & 0xffffu));
		a.dstzw_dy[3] = int(hi(w[11]) | lo16(w[15]));
	}

	// rdp_device.cpp:338-344
	static void decode_z(Attr &a, const uint32_t *w)
	{
		a.stzw[2] = int(w[0]);
		a.dstzw_dx[2] = int(w[1]);
		a.dstzw_de[2] = int(w[2]);
		a.dstzw_dy[2] = int(w[3]);
	}

	// ======================================================================= derived setup
	// rdp_renderer.cpp:717-740
	static int normalize_dzpix(int dz)
	{
		if (dz >= 0x8000) return 0x8000;
		if (dz == 0) return 1;
		int bit = 31 - __builtin_clz(uint32_t(dz));
		return 1 << (bit + 1);
	}
	static int dz_compress_host(int dz)
	{
		int v = 0;
		if (dz & 0xff00) v |= 8;
		if (dz & 0xf0f0) v |= 4;
		if (dz & 0xcccc) v |= 2;
		if (dz & 0xaaaa) v |= 1;
		return v;
	}

	// rdp_renderer.cpp:754-908: constant combiner inputs for one cycle.
	void build_combiner_constants(Derived &d, int cyc, const StaticState &st) const
	{
		auto rgb = [](int *o, uint32_t c) { o[0] = (c >> 24) & 0xff; o[1] = (c >> 16) & 0xff; o[2] = (c >> 8) & 0xff; };
		auto alp = [](int *o, uint32_t c) { o[3] = c & 0xff; };
		uint32_t prim = constants.primitive_color, env = constants.env_color;
		switch (st.rgb[cyc][0]) // muladd
		{
		case 5: rgb(d.c_muladd[cyc], env); break;
		case 3: rgb(d.c_muladd[cyc], prim); break;
		default: break;
		}
		switch (st.rgb[cyc][1]) // mulsub
		{
		case 5: rgb(d.c_mulsub[cyc], env); break;
		case 3: rgb(d.c_mulsub[cyc], prim); break;
		case 7: rgb(d.c_mulsub[cyc], uint32_t(constants.convert[4]) << 8); break;
		case 6:
			d.c_mulsub[cyc][0] = constants.key_center[0] & 0xff;
			d.c_mulsub[cyc][1] = constants.key_center[1] & 0xff;
			d.c_mulsub[cyc][2] = constants.key_center[2] & 0xff;
			break;
		default: break;
		}
		switch (st.rgb[cyc][2]) // mul
		{
		case 3: rgb(d.c_mul[cyc], prim); break;
		case 5: rgb(d.c_mul[cyc], env); break;
		case 10: rgb(d.c_mul[cyc], 0x01010101u * (prim & 0xff)); break;
		case 12: rgb(d.c_mul[cyc], 0x01010101u * (env & 0xff)); break;
		case 14: rgb(d.c_mul[cyc], 0x01010101u * uint32_t(constants.prim_lod_frac)); break;
		case 15: rgb(d.c_mul[cyc], uint32_t(constants.convert[5]) << 8); break;
		case 6:
			d.c_mul[cyc][0] = constants.key_scale[0] & 0xff;
			d.c_mul[cyc][1] = constants.key_scale[1] & 0xff;
			d.c_mul[cyc][2] = constants.key_scale[2] & 0xff;
			break;
		default: break;
		}
		switch (st.rgb[cyc][3]) // add
		{
		case 3: rgb(d.c_add[cyc], prim); break;
		case 5: rgb(d.c_add[cyc], env); break;
		default: break;
		}
		switch (st.alpha[cyc][0])
		{
		case 3: alp(d.c_muladd[cyc], prim); break;
		case 5: alp(d.c_muladd[cyc], env); break;
		default: break;
		}
		switch (st.alpha[cyc][1])
		{
		case 3: alp(d.c_mulsub[cyc], prim); break;
		case 5: alp(d.c_mulsub[cyc], env); break;
		default: break;
		}
		switch (st.alpha[cyc][2])
		{
		case 3: alp(d.c_mul[cyc], prim); break;
		case 5: alp(d.c_mul[cyc], env); break;
		case 6: alp(d.c_mul[cyc], uint32_t(constants.prim_lod_frac)); break;
		default: break;
		}
		switch (st.alpha[cyc][3])
		{
		case 3: alp(d.c_add[cyc], prim); break;
		case 5: alp(d.c_add[cyc], env); break;
		default: break;
		}
	}

	// rdp_renderer.cpp:910-948
	Derived build_derived(const Attr &attr) const
	{
		Derived d = {};
		if (constants.use_prim_depth)
		{
			d.dz = constants.prim_dz & 0xffff;
			d.dz_compressed = dz_compress_host(d.dz);
		}
		else
		{
			int dzdx = attr.dstzw_dx[2] >> 16;
			int dzdy = attr.dstzw_dy[2] >> 16;
			int dzpix = (dzdx < 0 ? (~dzdx & 0x7fff) : dzdx) + (dzdy < 0 ? (~dzdy & 0x7fff) : dzdy);
			dzpix = normalize_dzpix(dzpix);
			d.dz = dzpix & 0xffff;
			d.dz_compressed = dz_compress_host(dzpix);
		}
		build_combiner_constants(d, 0, static_state);
		build_combiner_constants(d, 1, static_state);
		for (int i = 0; i < 4; i++)
		{
			d.fog[i] = (constants.fog_color >> (24 - 8 * i)) & 0xff;
			d.blend[i] = (constants.blend_color >> (24 - 8 * i)) & 0xff;
		}
		d.fill_color = constants.fill_color;
		d.min_lod = constants.min_level & 0xff;
		for (int i = 0; i < 4; i++)
			d.factors[i] = int16_t(constants.convert[i]);
		return d;
	}

	// rdp_renderer.cpp:1062-1134
	static bool acc_texel0(const StaticState &s, int c)
	{
		return s.rgb[c][0] == 1 || s.rgb[c][1] == 1 || s.rgb[c][2] == 1 || s.rgb[c][3] == 1 || s.rgb[c][2] == 8 ||
		       s.alpha[c][0] == 1 || s.alpha[c][1] == 1 || s.alpha[c][2] == 1 || s.alpha[c][3] == 1;
	}
	static bool acc_texel1(const StaticState &s, int c)
	{
		return s.rgb[c][0] == 2 || s.rgb[c][1] == 2 || s.rgb[c][2] == 2 || s.rgb[c][3] == 2 || s.rgb[c][2] == 9 ||
		       s.alpha[c][0] == 2 || s.alpha[c][1] == 2 || s.alpha[c][2] == 2 || s.alpha[c][3] == 2;
	}
	static bool acc_lod_frac(const StaticState &s, int c) { return s.rgb[c][2] == 13 || s.alpha[c][2] == 0; }

	// rdp_renderer.cpp:1333-1400 (only the flag deduction affects results; the static
	// texture format override is always equal to the per-tile format it replaces).
	void deduce_static_texture_state()
	{
		auto &st = static_state;
		if (st.flags & R_FILL) return;
		if (st.flags & R_COPY) return;
		bool multi = (st.flags & R_MULTI_CYCLE) != 0;
		bool t0 = multi ? (acc_texel0(st, 0) || acc_texel1(st, 1)) : acc_texel0(st, 1);
		bool t1 = multi ? (acc_texel1(st, 0) || acc_texel0(st, 1)) : false;
		bool pt1 = !multi ? acc_texel1(st, 1) : false;
		bool lodf = multi ? (acc_lod_frac(st, 0) || acc_lod_frac(st, 1)) : false;
		if (t1 && (st.flags & R_CONVERT_ONE)) t0 = true;
		st.flags &= ~(R_USES_TEXEL0 | R_USES_TEXEL1 | R_USES_PIPELINED_TEXEL1 | R_USES_LOD);
		if (t0) st.flags |= R_USES_TEXEL0;
		if (t1) st.flags |= R_USES_TEXEL1;
		if (pt1) st.flags |= R_USES_PIPELINED_TEXEL1;
		if (lodf || (st.flags & R_TEX_LOD)) st.flags |= R_USES_LOD;
	}

	// rdp_renderer.cpp:1136-1169
	void deduce_noise_state()
	{
		auto &st = static_state;
		st.flags &= ~(R_NEED_NOISE | R_NEED_NOISE_DUAL);
		if ((st.dither & 3) == 2 || ((st.dither >> 2) & 3) == 2)
		{
			st.flags |= R_NEED_NOISE;
			return;
		}
		if (st.flags & (R_COPY | R_FILL)) return;
		if ((st.flags & R_MULTI_CYCLE) && st.rgb[0][0] == 7) st.flags |= R_NEED_NOISE;
		if (st.rgb[1][0] == 7) st.flags |= R_NEED_NOISE;
		if ((st.flags & R_MULTI_CYCLE) && st.rgb[0][0] == 7 && st.rgb[1][0] == 7) st.flags |= R_NEED_NOISE_DUAL;
		if ((st.flags & (R_ALPHA_TEST | R_ALPHA_TEST_DITHER)) == (R_ALPHA_TEST | R_ALPHA_TEST_DITHER))
			st.flags |= R_NEED_NOISE;
	}

	// rdp_renderer.cpp:1171-1331
	static int norm_muladd(int v) { return (v == 7 || v == 1 || v == 2 || v == 0 || v == 6 || v == 4) ? v : 8; }
	static int norm_mulsub(int v) { return (v == 0 || v == 1 || v == 2 || v == 4 || v == 7) ? v : 8; }
	static int norm_mul(int v)
	{
		return (v == 0 || v == 7 || v == 1 || v == 2 || v == 8 || v == 9 || v == 4 || v == 11 || v == 13 || v == 15) ? v : 16;
	}
	static int norm_add(int v) { return (v == 1 || v == 2 || v == 0 || v == 6 || v == 4) ? v : 7; }
	static int norm_aaddsub(int v) { return (v == 0 || v == 1 || v == 2 || v == 4 || v == 6) ? v : 7; }
	static int norm_amul(int v) { return (v == 0 || v == 1 || v == 2 || v == 4) ? v : 7; }

	static StaticState normalize_static_state(StaticState st)
	{
		if (st.flags & R_FILL)
		{
			StaticState r = {};
			r.flags = R_FILL;
			return r;
		}
		if (st.flags & R_COPY)
		{
			uint32_t f = st.flags & (R_COPY | R_TLUT | R_TLUT_TYPE | R_USES_TEXEL0 | R_STATIC_TEX | R_TEX_LOD |
			                         R_DETAIL | R_PERSPECTIVE | R_ALPHA_TEST);
			StaticState r = {};
			r.flags = f;
			return r;
		}
		if ((st.flags & (R_MULTI_CYCLE | R_USES_PIPELINED_TEXEL1)) == 0)
			st.flags &= ~(R_BILERP1 | R_CONVERT_ONE);
		for (int c = 0; c < 2; c++)
		{
			st.rgb[c][0] = norm_muladd(st.rgb[c][0]);
			st.rgb[c][1] = norm_mulsub(st.rgb[c][1]);
			st.rgb[c][2] = norm_mul(st.rgb[c][2]);
			st.rgb[c][3] = norm_add(st.rgb[c][3]);
			st.alpha[c][0] = norm_aaddsub(st.alpha[c][0]);
			st.alpha[c][1] = norm_aaddsub(st.alpha[c][1]);
			st.alpha[c][2] = norm_amul(st.alpha[c][2]);
			st.alpha[c][3] = norm_aaddsub(st.alpha[c][3]);
		}
		return st;
	}

	// ======================================================================= span setup
	// parallel-rdp/shaders/span_setup.comp:59-227; L is log2 of the upscaling factor (0 at 1x).
	static int quantize_x(int x)
	{
		int sticky = (x & 0xfff) != 0 ? 1 : 0;
		return (x >> 12) | sticky;
	}

	// interpolate_snapped (span_setup.comp:80-85): whole pixels step by the full derivative,
	// sub-pixels of an upscaled pixel by the derivative divided by the factor.
	static int interpolate_snapped(int d, int dy, int L)
	{
		return (dy >> L) * d + (dy & ((1 << L) - 1)) * (d >> L);
	}

	static Span span_setup(const TriSetup &s, const Attr &a, const Scissor &sc, int y, int L = 0)
	{
		const int S = 1 << L;
		Span sp = {};
		bool flip = (s.flags & TRI_FLIP) != 0;
		bool interlace_en = (s.flags & TRI_INTERLACE_FIELD) != 0;
		bool keep_odd = (s.flags & TRI_INTERLACE_KEEP_ODD) != 0;
		{
			bool do_offset = (s.flags & TRI_DO_OFFSET) != 0;
			bool skip_xfrac = (s.flags & TRI_SKIP_XFRAC) != 0;
			int y_base = (s.yh >> 2) * S;
			int dy = y - y_base;
			int xh = s.xh * S + dy * (s.dxhdy << 2);
			int drgba_diff[4] = {}, dstzw_diff[4] = {};
			if (do_offset)
			{
				xh += (S * 3) * s.dxhdy;
				for (int c = 0; c < 4; c++)
				{
					int deh = a.drgba_de[c] & ~0x1ff, dyh = a.drgba_dy[c] & ~0x1ff;
					drgba_diff[c] = deh - (deh >> 2) - dyh + (dyh >> 2);
					deh = a.dstzw_de[c] & ~0x1ff;
					dyh = a.dstzw_dy[c] & ~0x1ff;
					dstzw_diff[c] = deh - (deh >> 2) - dyh + (dyh >> 2);
				}
			}
			int base_x = xh >> 15;
			int xfrac = skip_xfrac ? 0 : ((xh >> 7) & 0xff);
			for (int c = 0; c < 4; c++)
			{
				int v = a.rgba[c] + interpolate_snapped(a.drgba_de[c], dy, L);
				sp.rgba[c] = ((v & ~0x1ff) + drgba_diff[c] - interpolate_snapped((a.drgba_dx[c] >> 8) & ~1, xfrac, L)) & ~0x3ff;
				v = a.stzw[c] + interpolate_snapped(a.dstzw_de[c], dy, L);
				sp.stzw[c] = ((v & ~0x1ff) + dstzw_diff[c] - interpolate_snapped((a.dstzw_dx[c] >> 8) & ~1, xfrac, L)) & ~0x3ff;
			}
			sp.base_x = base_x;
		}

		int yh_base = (s.yh & ~3) * S;
		int ym_base = s.ym * S;
		int ylo = std::max(s.yh, sc.ylo) * S;
		int yhi = std::min(s.yl, sc.yhi) * S;
		int xl4[4], xr4[4];
		bool invalid[4];
		for (int i = 0; i < 4; i++)
		{
			int ys = y * 4 + i;
			bool clip_y = ys < ylo || ys >= yhi;
			int xh = s.xh * S + (ys - yh_base) * s.dxhdy;
			int xm = s.xm * S + (ys - yh_base) * s.dxmdy;
			int xl = s.xl * S + (ys - ym_base) * s.dxldy;
			if (ys < S * s.ym) xl = xm;
			xl = bfe_s(xl, 27 + L);
			xh = bfe_s(xh, 27 + L);
			int xhs = quantize_x(xh), xls = quantize_x(xl);
			xl4[i] = flip ? xhs : xls;
			xr4[i] = flip ? xls : xhs;
			invalid[i] = (xl4[i] >> 1) > (xr4[i] >> 1);
			invalid[i] = invalid[i] || clip_y;
		}
		int lo_sc = S * (sc.xlo << 1), hi_sc = S * (sc.xhi << 1);
		bool all_over = true, all_under = true;
		for (int i = 0; i < 4; i++)
		{
			all_over = all_over && (std::min(xl4[i], xr4[i]) >= hi_sc);
			all_under = all_under && (std::max(xl4[i], xr4[i]) < lo_sc);
		}
		bool all_invalid = true;
		for (int i = 0; i < 4; i++)
		{
			int l = std::min(std::max(xl4[i], lo_sc), hi_sc);
			int r = std::min(std::max(xr4[i], lo_sc), hi_sc);
			if (invalid[i]) { l = 0xffff; r = 0; }
			sp.xleft[i] = l;
			sp.xright[i] = r;
			all_invalid = all_invalid && invalid[i];
		}
		int mn = std::min(std::min(sp.xleft[0], sp.xleft[1]), std::min(sp.xleft[2], sp.xleft[3]));
		int mx = std::max(std::max(sp.xright[0], sp.xright[1]), std::max(sp.xright[2], sp.xright[3]));
		sp.start_x = mn >> 3;
		sp.end_x = mx >> 3;
		sp.valid = !all_invalid && !all_over && !all_under;
		if (interlace_en && (((y >> L) & 1) != int(keep_odd)))
			sp.valid = false;
		// lodlength is stored as int16 in the span record.
		sp.lodlength = int16_t(flip ? (sp.end_x - sp.base_x) : (sp.base_x - sp.start_x));
		// The xleft/xright values are stored as 16-bit unsigned in the span record.
		for (int i = 0; i < 4; i++)
		{
			sp.xleft[i] &= 0xffff;
			sp.xright[i] &= 0xffff;
		}
		return sp;
	}

	// ======================================================================= binning
	// parallel-rdp/shaders/binning.h:58-144; S is the upscaling factor (1 at 1x).
	static void interpolate_xs(const TriSetup &s, const int ys[4], bool flip, int &rmin, int &rmax, int S = 1)
	{
		int64_t yh_base = int64_t(s.yh & ~3) * S;
		int64_t ym_base = int64_t(s.ym) * S;
		int xls[4], xrs[4];
		for (int i = 0; i < 4; i++)
		{
			int64_t xh = int64_t(S * s.xh) + int64_t(ys[i] - yh_base) * s.dxhdy;
			int64_t xm = int64_t(S * s.xm) + int64_t(ys[i] - yh_base) * s.dxmdy;
			int64_t xl = int64_t(S * s.xl) + int64_t(ys[i] - ym_base) * s.dxldy;
			if (ys[i] < S * s.ym) xl = xm;
			auto sat = [](int64_t v) -> int {
				if (v > INT32_MAX) return INT32_MAX;
				if (v < INT32_MIN) return INT32_MIN;
				return int(v);
			};
			// The shader computes a 64-bit product and saturates on the high word.
			int xh32 = sat(xh), xl32 = sat(xl);
			int xhs = xh32 >> 15, xlsf = xl32 >> 15;
			xls[i] = flip ? xhs : xlsf;
			xrs[i] = flip ? xlsf : xhs;
		}
		int max_range = 0;
		for (int i = 0; i < 4; i++)
			max_range = std::max(max_range, std::max(std::abs(xls[i]), std::abs(xrs[i])));
		if (max_range <= 2047 * S)
		{
			rmin = std::min(std::min(xls[0], xls[1]), std::min(xls[2], xls[3]));
			rmax = std::max(std::max(xrs[0], xrs[1]), std::max(xrs[2], xrs[3]));
		}
		else
		{
			rmin = 0;
			rmax = 0x7fffffff;
		}
	}

	static bool bin_primitive(const TriSetup &s, int lox, int loy, int hix, int hiy, const Scissor &sc, int S = 1)
	{
		loy = std::max(loy, S * (sc.ylo >> 2));
		hiy = std::min(hiy, S * ((sc.yhi + 3) >> 2) - 1);
		int start_y = loy * 4;
		int end_y = hiy * 4 + 3;
		start_y = std::max(start_y, S * s.yh);
		end_y = std::min(end_y, S * s.yl - 1);
		if (end_y < start_y) return false;
		bool flip = (s.flags & TRI_FLIP) != 0;
		int ys[4] = { start_y, end_y, clampi(S * s.ym - 1, start_y, end_y), clampi(S * s.ym, start_y, end_y) };
		int rx0, rx1;
		interpolate_xs(s, ys, flip, rx0, rx1, S);
		int x_bias = (s.flags & TRI_FILL_COPY_RASTER) ? 4 : 3;
		int sx0 = S * (sc.xlo >> 2), sx1 = S * ((sc.xhi + x_bias) >> 2) - 1;
		rx0 = clampi(rx0, sx0, sx1);
		rx1 = clampi(rx1, sx0, sx1);
		rx0 = std::max(rx0, lox);
		rx1 = std::min(rx1, hix);
		return rx0 <= rx1;
	}

	// ======================================================================= noise / dither
	void reseed_noise(uint32_t x, uint32_t y, uint32_t p)
	{
		const uint32_t P = 1103515245u;
		uint32_t s0 = x, s1 = y, s2 = p;
		for (int i = 0; i < 3; i++)
		{
			uint32_t n0 = ((s0 >> 8) ^ s1) * P;
			uint32_t n1 = ((s1 >> 8) ^ s2) * P;
			uint32_t n2 = ((s2 >> 8) ^ s0) * P;
			s0 = n0; s1 = n1; s2 = n2;
		}
		seeded_noise = (s0 >> 16) & 0xffff;
	}
	int noise_combiner() const { return int(((seeded_noise & 7u) << 6) | 0x20u); }
	int noise_dither_alpha() const { return int(seeded_noise & 7u); }
	int noise_dither_color() const { return int(seeded_noise & 0x1ffu); }
	int noise_blend_threshold() const { return int(seeded_noise & 0xffu); }

	void dither_coefficients(int x, int y, int mode_rgb, int mode_alpha, int &rgb_d, int &alpha_d) const
	{
		const int SPLAT = 1 | 8 | 64;
		if (mode_rgb < 2) rgb_d = dither_matrices[mode_rgb][(y & 3) * 4 + (x & 3)] * SPLAT;
		else if (mode_rgb == 2) rgb_d = noise_dither_color();
		else rgb_d = 0;
		if (mode_alpha == 3) alpha_d = 0;
		else if (mode_alpha == 2) alpha_d = noise_dither_alpha();
		else
		{
			alpha_d = mode_rgb >= 2 ? dither_matrices[mode_rgb & 1][(y & 3) * 4 + (x & 3)] : (rgb_d & 7);
			if (mode_alpha == 1) alpha_d = ~alpha_d & 7;
		}
	}

	static void rgb_dither(int rgb[3], int dith)
	{
		for (int c = 0; c < 3; c++)
		{
			int d = (dith >> (3 * c)) & 7;
			int o = rgb[c];
			int r = o > 247 ? 255 : ((o & 0xf8) + 8);
			int replace_sign = (d - (o & 7)) >> 31;
			int diff = r - o;
			rgb[c] = (o + (diff & replace_sign)) & 0xff;
		}
	}

	// ======================================================================= clamping / interpolation
	static int clamp_9bit_notrunc(int c) { return clampi(bfe_s(c - 0x80, 9) + 0x80, 0, 0xff); }
	static int clamp_z(int z)
	{
		z -= 1 << 17;
		z = int(uint32_t(z) << 13) >> 13;
		z += 1 << 17;
		return clampi(z, 0, 0x3ffff);
	}

	// interpolation.h:29-53.  The 16-bit snapped value of the shader keeps every bit this reads.
	static void interpolate_rgba(const int rgba_in[4], const int ddx[4], const int ddy[4], int dx, int coverage, int out[4],
	                             int L = 0)
	{
		int first = find_lsb(uint32_t(coverage));
		int yoff = first >> 1;
		int xoff = ((first & 1) << 1) + (yoff & 1);
		for (int c = 0; c < 4; c++)
		{
			int v = rgba_in[c] + ((ddx[c] & ~0x1f) >> L) * dx;
			int sn = v >> 14;
			sn <<= 2 + L;
			sn += xoff * (ddx[c] >> 14) + yoff * (ddy[c] >> 14);
			sn >>= 4 + L;
			out[c] = clamp_9bit_notrunc(sn);
		}
	}

	static void perspective_get_lut(int w, int &rcp, int &shift)
	{
		shift = std::min(14 - find_msb(w), 14);
		int normout = (w << shift) & 0x3fff;
		int wnorm = normout & 0xff;
		int idx = normout >> 8;
		rcp = ((-int(persp_slope[idx]) * 4 * wnorm) >> 10) + persp_base[idx];
	}

	static void perspective_divide(const int stw[3], int st[2], bool &overflow)
	{
		int w = stw[2];
		bool w_carry = w <= 0;
		w &= 0x7fff;
		int rcp, shift;
		perspective_get_lut(w, rcp, shift);
		int prod[2] = { stw[0] * rcp, stw[1] * rcp };
		int temp_mask = ((1 << 30) - 1) & -((1 << 29) >> shift);
		int oob[2] = { prod[0] & temp_mask, prod[1] & temp_mask };
		int temp[2];
		for (int i = 0; i < 2; i++)
		{
			if (shift != 14) temp[i] = prod[i] = prod[i] >> (13 - shift);
			else temp[i] = prod[i] << 1;
		}
		if (oob[0] != 0 || oob[1] != 0)
		{
			for (int i = 0; i < 2; i++)
			{
				if (oob[i] != temp_mask && oob[i] != 0)
				{
					temp[i] = (prod[i] & (1 << 29)) == 0 ? 0x7fff : -0x8000;
					overflow = true;
				}
			}
		}
		if (w_carry)
		{
			temp[0] = temp[1] = 0x7fff;
			overflow = true;
		}
		st[0] = clampi(temp[0], -0x10000, 0xffff);
		st[1] = clampi(temp[1], -0x10000, 0xffff);
	}

	static void st_divide(const int stw[3], bool perspective, int st[2], bool &overflow)
	{
		if (perspective) perspective_divide(stw, st, overflow);
		else { st[0] = stw[0]; st[1] = stw[1]; }
	}

	void interpolate_st_copy(const Span &sp, const int dstzw_dx[4], int x, bool perspective, bool flip,
	                         int dx_mask, int dx_shift, int st[2], int &s_offset, int L = 0) const
	{
		int dx = flip ? (x - sp.start_x) : (sp.end_x - x);
		// Upscaled copies repeat pixels (interpolation.h:60-61).
		dx >>= L;
		int snapped = dx & dx_mask;
		s_offset = dx - snapped;
		int lerp_dx = (dx >> dx_shift) * (flip ? 1 : -1);
		int stw[3] = { (sp.stzw[0] + (dstzw_dx[0] & ~0x1f) * lerp_dx) >> 16,
		               (sp.stzw[1] + (dstzw_dx[1] & ~0x1f) * lerp_dx) >> 16,
		               (sp.stzw[3] + (dstzw_dx[3] & ~0x1f) * lerp_dx) >> 16 };
		bool ov = false;
		st_divide(stw, perspective, st, ov);
	}

	static void interpolate_st_single(const int stzw[4], const int dstzw_dx[4], int dx, bool perspective, int st[2],
	                                  int L = 0)
	{
		int stw[3] = { (stzw[0] + ((dstzw_dx[0] & ~0x1f) >> L) * dx) >> 16,
		               (stzw[1] + ((dstzw_dx[1] & ~0x1f) >> L) * dx) >> 16,
		               (stzw[3] + ((dstzw_dx[3] & ~0x1f) >> L) * dx) >> 16 };
		bool ov = false;
		st_divide(stw, perspective, st, ov);
	}

	// interpolation.h:93-141.
	static void interpolate_stz(const int stzw[4], const int ddx[4], const int ddy[4], int dx, int coverage,
	                            bool perspective, bool uses_lod, int flip_dir, int st[2], int st_dx[2], int st_dy[2],
	                            int &z, bool &overflow, int L = 0)
	{
		const int S = 1 << L;
		int idx[3] = { 0, 1, 3 };
		int stw[3], stw_dx[3], stw_dy[3];
		for (int i = 0; i < 3; i++)
		{
			int c = idx[i];
			stw[i] = stzw[c] + ((ddx[c] & ~0x1f) >> L) * dx;
		}
		if (uses_lod)
		{
			for (int i = 0; i < 3; i++)
			{
				int c = idx[i];
				stw_dx[i] = stw[i] + flip_dir * ((ddx[c] & ~0x1f) >> L);
				stw_dy[i] = stw[i] + (S > 1 ? std::abs(flip_dir) : 1) * ((ddy[c] & ~0x7fff) >> L);
			}
		}
		int s0[3] = { stw[0] >> 16, stw[1] >> 16, stw[2] >> 16 };
		st_divide(s0, perspective, st, overflow);
		if (uses_lod)
		{
			int s1[3] = { stw_dx[0] >> 16, stw_dx[1] >> 16, stw_dx[2] >> 16 };
			int s2[3] = { stw_dy[0] >> 16, stw_dy[1] >> 16, stw_dy[2] >> 16 };
			st_divide(s1, perspective, st_dx, overflow);
			st_divide(s2, perspective, st_dy, overflow);
		}
		z = stzw[2] + ddx[2] * (dx >> L) + (ddx[2] >> L) * (dx & (S - 1));
		int sz = z >> 10;
		int first = find_lsb(uint32_t(coverage));
		int yoff = first >> 1;
		int xoff = ((first & 1) << 1) + (yoff & 1);
		sz <<= 2 + L;
		sz += xoff * (ddx[2] >> 10) + yoff * (ddy[2] >> 10);
		sz >>= 5 + L;
		z = clamp_z(sz);
	}

	// ======================================================================= coverage
	static int compute_coverage(const int xl[4], const int xr[4], int x)
	{
		int xs = (x << 3) & 0xffff;
		static const int offs[4] = { 0, 4, 2, 6 };
		int clip = 0;
		// Sample (i, j): sub-scanline i in {0..3}, x offset from offs; bit layout from coverage.h:33-43.
		for (int k = 0; k < 4; k++)
		{
			int xsh = (xs + offs[k]) & 0xffff;
			// clip_x0 uses xleft.xxyy / xright.xxyy: components k -> line (k>>1)
			int l0 = k >> 1;
			int l1 = 2 + (k >> 1);
			bool c0 = xsh < xl[l0] || xsh >= xr[l0];
			bool c1 = xsh < xl[l1] || xsh >= xr[l1];
			if (c0) clip |= 1 << k;
			if (c1) clip |= 16 << k;
		}
		return ~clip & 0xff;
	}

	static int blend_coverage(int coverage, int memory_coverage, bool blend_en, int mode)
	{
		switch (mode)
		{
		case 0: return blend_en ? std::min(7, memory_coverage + coverage) : ((coverage - 1) & 7);
		case 1: return (coverage + memory_coverage) & 7;
		case 2: return 7;
		default: return memory_coverage;
		}
	}

	// ======================================================================= texture
	static int texel_mask_s(const TileInfo &t, int s)
	{
		if (t.mask_s != 0)
		{
			int mask = 1 << t.mask_s;
			if (t.flags & TILE_MIRROR_S) s ^= std::max((s & mask) - 1, 0);
			s &= mask - 1;
		}
		return s;
	}
	static int texel_mask_t(const TileInfo &t, int v)
	{
		if (t.mask_t != 0)
		{
			int mask = 1 << t.mask_t;
			if (t.flags & TILE_MIRROR_T) v ^= std::max((v & mask) - 1, 0);
			v &= mask - 1;
		}
		return v;
	}

	struct T4 { int v[4]; };

	static T4 convert_rgba16(uint32_t w)
	{
		T4 r;
		for (int c = 0; c < 3; c++)
		{
			uint32_t x = (w >> (11 - 5 * c)) & 31u;
			r.v[c] = int((x << 3) | (x >> 2));
		}
		r.v[3] = int((w & 1u) * 0xffu);
		return r;
	}
	static T4 convert_ia16(uint32_t w)
	{
		int i = int(w >> 8), a = int(w & 0xff);
		return { { i, i, i, a } };
	}
	static T4 splat(int v) { return { { v, v, v, v } }; }

	uint32_t byte_index(const TileInfo &t, int s_bytes, int tv, uint32_t wrap) const
	{
		uint32_t off = (t.offset + t.stride * uint32_t(tv) + uint32_t(s_bytes)) & wrap;
		off ^= (uint32_t(tv) & 1u) << 2;
		off ^= 3u;
		return off;
	}
	uint32_t hw_index(const TileInfo &t, int s, int tv, uint32_t wrap) const
	{
		uint32_t off = (t.offset + t.stride * uint32_t(tv) + uint32_t(s) * 2u) & wrap;
		uint32_t idx = off >> 1;
		idx ^= (uint32_t(tv) & 1u) << 1;
		idx ^= 1u;
		return idx;
	}

	T4 texel_rgba4(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		uint32_t idx = byte_index(t, s >> 1, tv, 0xfff);
		uint32_t shift = (~uint32_t(s) & 1u) * 4;
		uint32_t w = (tm8(tm, idx) >> shift) & 0xf;
		w |= w << 4;
		return splat(int(w));
	}
	T4 texel_ia4(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		uint32_t idx = byte_index(t, s >> 1, tv, 0xfff);
		uint32_t shift = (~uint32_t(s) & 1u) * 4;
		uint32_t w = (tm8(tm, idx) >> shift) & 0xf;
		uint32_t i = w & 0xe;
		i = (i << 4) | (i << 1) | (i >> 2);
		return { { int(i), int(i), int(i), int((w & 1) * 0xff) } };
	}
	T4 texel_ci4(const uint16_t *tm, const TileInfo &t, int s, int tv, uint32_t pal) const
	{
		uint32_t idx = byte_index(t, s >> 1, tv, 0xfff);
		uint32_t shift = (~uint32_t(s) & 1u) * 4;
		uint32_t w = (tm8(tm, idx) >> shift) & 0xf;
		w |= pal << 4;
		return splat(int(w));
	}
	T4 texel_ci4_tlut(const uint16_t *tm, const TileInfo &t, int s, int tv, uint32_t pal, uint32_t lut_off,
	                  uint32_t addr_xor, bool tlut_type) const
	{
		uint32_t idx = byte_index(t, s >> 1, tv, 0x7ff);
		uint32_t shift = (~uint32_t(s) & 1u) * 4;
		uint32_t w = (tm8(tm, idx) >> shift) & 0xf;
		w |= pal << 4;
		uint32_t e = ((w << 2) + lut_off) ^ addr_xor;
		w = tm[(0x400 | e) & 2047];
		return tlut_type ? convert_ia16(w) : convert_rgba16(w);
	}
	T4 texel_ci8_tlut(const uint16_t *tm, const TileInfo &t, int s, int tv, uint32_t lut_off, uint32_t addr_xor,
	                  bool tlut_type) const
	{
		uint32_t idx = byte_index(t, s, tv, 0x7ff);
		uint32_t w = tm8(tm, idx);
		uint32_t e = ((w << 2) + lut_off) ^ addr_xor;
		w = tm[(0x400 | e) & 2047];
		return tlut_type ? convert_ia16(w) : convert_rgba16(w);
	}
	T4 texel_ci32(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		uint32_t w = tm[hw_index(t, s, tv, 0xfff) & 2047];
		int a = int(w >> 8), b = int(w & 0xff);
		return { { a, b, a, b } };
	}
	T4 texel_ci32_tlut(const uint16_t *tm, const TileInfo &t, int s, int tv, uint32_t lut_off, uint32_t addr_xor,
	                   bool tlut_type) const
	{
		uint32_t w = tm[hw_index(t, s, tv, 0x7ff) & 2047];
		uint32_t e = (((w >> 6) & ~3u) + lut_off) ^ addr_xor;
		w = tm[(0x400 | e) & 2047];
		return tlut_type ? convert_ia16(w) : convert_rgba16(w);
	}
	T4 texel_rgba8(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		return splat(tm8(tm, byte_index(t, s, tv, 0xfff)));
	}
	T4 texel_ia8(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		uint32_t w = tm8(tm, byte_index(t, s, tv, 0xfff));
		uint32_t i = w >> 4, a = w & 0xf;
		a |= a << 4;
		i |= i << 4;
		return { { int(i), int(i), int(i), int(a) } };
	}
	T4 texel_yuv16(const uint16_t *tm, const TileInfo &t, int s, int tv, uint32_t chroma_x) const
	{
		uint32_t base = t.offset + t.stride * uint32_t(tv);
		uint32_t ol = (base + uint32_t(s)) & 0x7ff;
		uint32_t oc = (base + chroma_x * 2) & 0x7ff;
		uint32_t il = (ol ^ ((uint32_t(tv) & 1u) << 2)) ^ 3u;
		uint32_t ic = ((oc >> 1) ^ ((uint32_t(tv) & 1u) << 1)) ^ 1u;
		int luma = tm8(tm, il | 0x800);
		uint32_t chroma = tm[ic & 2047];
		int u = int((chroma >> 8) & 0xff), v = int(chroma & 0xff);
		return { { u - 0x80, v - 0x80, luma, luma } };
	}
	T4 texel_rgba16(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		return convert_rgba16(tm[hw_index(t, s, tv, 0xfff) & 2047]);
	}
	T4 texel_ia16(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		return convert_ia16(tm[hw_index(t, s, tv, 0xfff) & 2047]);
	}
	T4 texel_rgba32(const uint16_t *tm, const TileInfo &t, int s, int tv) const
	{
		uint32_t idx = hw_index(t, s, tv, 0x7ff) & 2047;
		uint32_t lo = tm[idx], hi = tm[(idx | 0x400) & 2047];
		return { { int(lo >> 8), int(lo & 0xff), int(hi >> 8), int(hi & 0xff) } };
	}

	static int clamp_and_shift_coord(bool clamp_bit, int coord, int lo, int hi, int shift)
	{
		coord = clampi(coord, -0x8000, 0x7fff);
		if (shift < 11) coord >>= shift;
		else
		{
			coord = int(uint32_t(coord) << (32 - shift));
			coord >>= 16;
		}
		if (clamp_bit)
		{
			bool clamp_hi = (coord >> 3) >= hi;
			if (clamp_hi) coord = (((hi >> 2) - (lo >> 2)) & 0x3ff) << 5;
			else coord = std::max(coord - (lo << 3), 0);
		}
		else
			coord -= lo << 3;
		return coord;
	}

	static int shift_coord(int coord, int lo, int shift)
	{
		coord = clampi(coord, -0x8000, 0x7fff);
		if (shift < 11) coord >>= shift;
		else
		{
			coord = int(uint32_t(coord) << (32 - shift));
			coord >>= 16;
		}
		return coord - (lo << 3);
	}

	int sample_texture_copy_word(const uint16_t *tm, const TileInfo &t, int st0, int st1, int s_offset, bool tlut) const
	{
		bool high_word = s_offset < 2;
		bool replicate_8bpp = high_word && t.size != 2 && !tlut;
		int s_shamt = std::min(t.size, 2);
		bool large_texel = t.size == 3;
		uint32_t idx_mask = (large_texel || tlut) ? 0x3ffu : 0x7ffu;
		int samp;
		if (replicate_8bpp)
		{
			st0 += 2 * s_offset;
			int sa = st0, sb = st0 + 1;
			if (t.mask_s != 0)
			{
				int mask = 1 << t.mask_s;
				if (t.flags & TILE_MIRROR_S)
				{
					sa ^= std::max((sa & mask) - 1, 0);
					sb ^= std::max((sb & mask) - 1, 0);
				}
				sa &= mask - 1;
				sb &= mask - 1;
			}
			int tv = texel_mask_t(t, st1);
			uint32_t tbase = t.offset + t.stride * uint32_t(tv);
			uint32_t na = (tbase * 2 + (uint32_t(sa) << s_shamt)) & 0x1fffu;
			uint32_t nb = (tbase * 2 + (uint32_t(sb) << s_shamt)) & 0x1fffu;
			na ^= (uint32_t(tv) & 1u) * 8u;
			nb ^= (uint32_t(tv) & 1u) * 8u;
			uint32_t ia = (na >> 2) & idx_mask, ib = (nb >> 2) & idx_mask;
			int s0 = tm[(ia ^ 1) & 2047];
			int s1 = tm[(ib ^ 1) & 2047];
			if (t.size == 1)
			{
				s0 >>= 8 - 4 * int(na & 2);
				s1 >>= 8 - 4 * int(nb & 2);
				s0 &= 0xff;
				s1 &= 0xff;
			}
			else if (t.size == 0)
			{
				s0 >>= 12 - 4 * int(na & 3u);
				s1 >>= 12 - 4 * int(nb & 3u);
				s0 = (s0 & 0xf) * 0x11;
				s1 = (s1 & 0xf) * 0x11;
			}
			else
			{
				s0 >>= 8;
				s1 >>= 8;
			}
			samp = (s0 << 8) | s1;
		}
		else
		{
			st0 += s_offset;
			int s = texel_mask_s(t, st0);
			int tv = texel_mask_t(t, st1);
			uint32_t tbase = t.offset + t.stride * uint32_t(tv);
			uint32_t nib = (tbase * 2 + (uint32_t(s) << s_shamt)) & 0x1fffu;
			nib ^= (uint32_t(tv) & 1u) * 8u;
			uint32_t idx = (nib >> 2) & idx_mask;
			samp = tm[(idx ^ 1) & 2047];
			if (tlut)
			{
				if (t.size == 0)
				{
					samp >>= 12 - 4 * int(nib & 3);
					samp &= 0xf;
					samp |= t.palette << 4;
					samp <<= 2;
					samp += s_offset;
				}
				else
				{
					samp >>= 8 - 4 * int(nib & 2);
					samp &= 0xff;
					samp <<= 2;
					samp += s_offset;
				}
				samp = tm[((uint32_t(samp) | 0x400u) ^ 1u) & 2047];
			}
		}
		return samp;
	}

	int sample_texture_copy(const uint16_t *tm, const TileInfo &t, int st0, int st1, int s_offset, bool tlut,
	                        int fb_size) const
	{
		st0 = shift_coord(st0, int(t.slo), t.shift_s);
		st1 = shift_coord(st1, int(t.tlo), t.shift_t);
		st0 >>= 5;
		st1 >>= 5;
		if (fb_size == 0) return 0;
		if (fb_size == 1)
		{
			int samp = sample_texture_copy_word(tm, t, st0, st1, s_offset >> 1, tlut);
			samp >>= 8 - 8 * (s_offset & 1);
			return samp & 0xff;
		}
		return sample_texture_copy_word(tm, t, st0, st1, s_offset, tlut);
	}

	static T4 texture_convert_factors(const T4 &tin, const int f[4])
	{
		int tx[4];
		for (int i = 0; i < 4; i++) tx[i] = bfe_s(tin.v[i], 9);
		int r = tx[2] + ((f[0] * tx[1] + 0x80) >> 8);
		int g = tx[2] + ((f[1] * tx[0] + f[2] * tx[1] + 0x80) >> 8);
		int b = tx[2] + ((f[3] * tx[0] + 0x80) >> 8);
		return { { r, g, b, tx[2] } };
	}

	static void bilinear_3tap2(const int *tb, const int *t10, const int *t01, const int *t11, int fx, int fy, int *out)
	{
		int sum = fx + fy;
		const int *base = sum >= 32 ? t11 : tb;
		int ffx = sum >= 32 ? 32 - fy : fx;
		int ffy = sum >= 32 ? 32 - fx : fy;
		for (int i = 0; i < 2; i++)
		{
			int acc = (t10[i] - base[i]) * ffx;
			acc += (t01[i] - base[i]) * ffy;
			acc += 0x10;
			acc >>= 5;
			out[i] = acc + base[i];
		}
	}

	// texture.h:498-923
	T4 sample_texture(const uint16_t *tm, const TileInfo &t, int st0, int st1, bool tlut, bool tlut_type,
	                  bool sample_quad, bool mid_texel_state, bool convert_one, bool bilerp, const int factors[4],
	                  const T4 &prev) const
	{
		st0 = clamp_and_shift_coord((t.flags & TILE_CLAMP_S) != 0, st0, int(t.slo), int(t.shi), t.shift_s);
		st1 = clamp_and_shift_coord((t.flags & TILE_CLAMP_T) != 0, st1, int(t.tlo), int(t.thi), t.shift_t);
		int fx = 0, fy = 0;
		if (sample_quad || tlut) { fx = st0 & 31; fy = st1 & 31; }
		int sum_frac = fx + fy;
		st0 >>= 5;
		st1 >>= 5;
		int s0 = texel_mask_s(t, st0);
		int t0 = texel_mask_t(t, st1);
		int s1 = texel_mask_s(t, st0 + 1);
		int t1 = texel_mask_t(t, st1 + 1);
		int tdiff = std::max(t1 - t0, -255);
		t1 = (t0 & 0xff) + tdiff;
		t0 &= 0xff;

		T4 tb = {}, t10 = {}, t01 = {}, t11 = {};
		bool mid_texel = mid_texel_state && bilerp && fx == 0x10 && fy == 0x10;
		bool upper_lut = sum_frac >= 0x20;
		if (mid_texel) sum_frac = 0;
		bool yuv = t.fmt == FMT_YUV;
		int bs = sum_frac >= 0x20 ? s1 : s0;
		int bt = sum_frac >= 0x20 ? t1 : t0;
		int chroma_frac = ((s0 & 1) << 4) | (fx >> 1);

		if (tlut)
		{
			if (!sample_quad)
			{
				bs = s0;
				bt = t0;
				s1 = s0;
				t1 = t0;
			}
			switch (t.fmt)
			{
			case FMT_RGBA: case FMT_CI: case FMT_IA: case FMT_I:
			{
				bool upper = sum_frac >= 0x20;
				uint32_t ax = upper_lut ? 2 : 1;
				uint32_t pal = uint32_t(t.palette);
				switch (t.size)
				{
				case 0:
					tb = texel_ci4_tlut(tm, t, bs, bt, pal, upper ? 3 : 0, ax, tlut_type);
					if (bilerp)
					{
						t10 = texel_ci4_tlut(tm, t, s1, t0, pal, 1, ax, tlut_type);
						t01 = texel_ci4_tlut(tm, t, s0, t1, pal, 2, ax, tlut_type);
					}
					if (mid_texel) t11 = texel_ci4_tlut(tm, t, s1, t1, pal, 3, ax, tlut_type);
					break;
				case 1:
					tb = texel_ci8_tlut(tm, t, bs, bt, upper ? 3 : 0, ax, tlut_type);
					if (bilerp)
					{
						t10 = texel_ci8_tlut(tm, t, s1, t0, 1, ax, tlut_type);
						t01 = texel_ci8_tlut(tm, t, s0, t1, 2, ax, tlut_type);
					}
					if (mid_texel) t11 = texel_ci8_tlut(tm, t, s1, t1, 3, ax, tlut_type);
					break;
				default:
					tb = texel_ci32_tlut(tm, t, bs, bt, upper ? 3 : 0, ax, tlut_type);
					if (bilerp)
					{
						t10 = texel_ci32_tlut(tm, t, s1, t0, 1, ax, tlut_type);
						t01 = texel_ci32_tlut(tm, t, s0, t1, 2, ax, tlut_type);
					}
					if (mid_texel) t11 = texel_ci32_tlut(tm, t, s1, t1, 3, ax, tlut_type);
					break;
				}
				break;
			}
			default:
				break; // YUV with TLUT leaves the texels undefined in the reference; we use zero.
			}
		}
		else
		{
			auto fetch = [&](int s, int tv) -> T4 {
				switch (t.fmt)
				{
				case FMT_RGBA:
					switch (t.size)
					{
					case 0: return texel_rgba4(tm, t, s, tv);
					case 1: return texel_rgba8(tm, t, s, tv);
					case 2: return texel_rgba16(tm, t, s, tv);
					default: return texel_rgba32(tm, t, s, tv);
					}
				case FMT_CI:
					switch (t.size)
					{
					case 0: return texel_ci4(tm, t, s, tv, uint32_t(t.palette));
					case 1: return texel_rgba8(tm, t, s, tv);
					default: return texel_ci32(tm, t, s, tv);
					}
				case FMT_IA:
					switch (t.size)
					{
					case 0: return texel_ia4(tm, t, s, tv);
					case 1: return texel_ia8(tm, t, s, tv);
					case 2: return texel_ia16(tm, t, s, tv);
					default: return texel_ci32(tm, t, s, tv);
					}
				case FMT_I:
					switch (t.size)
					{
					case 0: return texel_rgba4(tm, t, s, tv);
					case 1: return texel_rgba8(tm, t, s, tv);
					default: return texel_ci32(tm, t, s, tv);
					}
				default:
					return T4{};
				}
			};
			if (yuv)
			{
				uint32_t cx0 = uint32_t(s0 >> 1);
				uint32_t cx1 = uint32_t((s1 + (s1 - s0)) >> 1);
				tb = texel_yuv16(tm, t, s0, t0, cx0);
				if (sample_quad)
				{
					t10 = texel_yuv16(tm, t, s1, t0, cx1);
					t01 = texel_yuv16(tm, t, s0, t1, cx0);
					t11 = texel_yuv16(tm, t, s1, t1, cx1);
				}
			}
			else if (t.fmt <= FMT_I)
			{
				tb = fetch(bs, bt);
				if (sample_quad)
				{
					t10 = fetch(s1, t0);
					t01 = fetch(s0, t1);
				}
				if (mid_texel) t11 = fetch(s1, t1);
			}
		}

		T4 acc;
		if (convert_one)
		{
			int ps[4];
			for (int i = 0; i < 4; i++) ps[i] = bfe_s(prev.v[i], 9);
			if (sample_quad)
			{
				bool mid_rg = yuv ? (mid_texel_state && chroma_frac == 0x10 && fy == 0x10) : mid_texel;
				bool mid_ba = mid_texel;
				bool upper_ba = sum_frac >= 32;
				bool upper_rg = yuv ? ((chroma_frac + fy) >= 32 && !mid_rg) : upper_ba;
				int frg[2] = { upper_rg ? ps[1] : ps[0], upper_rg ? ps[0] : ps[1] };
				int fba[2] = { upper_ba ? ps[1] : ps[0], upper_ba ? ps[0] : ps[1] };
				int conv[4];
				for (int i = 0; i < 2; i++)
				{
					if (mid_rg)
						conv[i] = frg[0] * (t01.v[i] - t11.v[i]) + frg[1] * (t10.v[i] - t11.v[i]) +
						          ((tb.v[i] - t11.v[i]) << 6) + 0x80;
					else
					{
						int base = (upper_rg && yuv) ? t11.v[i] : tb.v[i];
						conv[i] = frg[0] * (t10.v[i] - base) + frg[1] * (t01.v[i] - base) + 0x80;
					}
				}
				for (int i = 2; i < 4; i++)
				{
					if (mid_ba)
						conv[i] = fba[0] * (t01.v[i] - t11.v[i]) + fba[1] * (t10.v[i] - t11.v[i]) +
						          ((tb.v[i] - t11.v[i]) << 6) + 0x80;
					else
					{
						int base = (upper_ba && yuv) ? t11.v[i] : tb.v[i];
						conv[i] = fba[0] * (t10.v[i] - base) + fba[1] * (t01.v[i] - base) + 0x80;
					}
				}
				for (int i = 0; i < 4; i++) acc.v[i] = (conv[i] >> 8) + ps[2];
			}
			else
				acc = splat(ps[2]);
		}
		else if (yuv)
		{
			if (sample_quad)
			{
				int ch[2], lu[2];
				if (bilerp)
				{
					bool mid_chroma = mid_texel_state && chroma_frac == 0x10 && fy == 0x10;
					if (mid_chroma)
						for (int i = 0; i < 2; i++) ch[i] = (tb.v[i] + t10.v[i] + t11.v[i] + t01.v[i] + 2) >> 2;
					else
						bilinear_3tap2(tb.v, t10.v, t01.v, t11.v, chroma_frac, fy, ch);
					if (mid_texel)
						for (int i = 0; i < 2; i++) lu[i] = (tb.v[2 + i] + t10.v[2 + i] + t11.v[2 + i] + t01.v[2 + i] + 2) >> 2;
					else
						bilinear_3tap2(tb.v + 2, t10.v + 2, t01.v + 2, t11.v + 2, fx, fy, lu);
				}
				else
				{
					for (int i = 0; i < 2; i++)
					{
						lu[i] = (fx + fy >= 32) ? t11.v[2 + i] : tb.v[2 + i];
						ch[i] = (chroma_frac + fy >= 32) ? t11.v[i] : tb.v[i];
					}
				}
				acc = { { ch[0], ch[1], lu[0], lu[1] } };
			}
			else
				acc = tb;
		}
		else if (mid_texel)
		{
			for (int i = 0; i < 4; i++) acc.v[i] = (tb.v[i] + t01.v[i] + t10.v[i] + t11.v[i] + 2) >> 2;
		}
		else if (bilerp && (sample_quad || tlut))
		{
			int ffx = sum_frac >= 32 ? 32 - fy : fx;
			int ffy = sum_frac >= 32 ? 32 - fx : fy;
			for (int i = 0; i < 4; i++)
			{
				int a = (t10.v[i] - tb.v[i]) * ffx;
				a += (t01.v[i] - tb.v[i]) * ffy;
				a += 0x10;
				a >>= 5;
				acc.v[i] = a + tb.v[i];
			}
		}
		else
			acc = tb;

		if (!bilerp && !convert_one) acc = texture_convert_factors(acc, factors);
		return acc;
	}

	// texture.h:925-1003
	static void compute_lod_2cycle(uint32_t &tile0, uint32_t &tile1, int &lod_frac, uint32_t max_level, int min_lod,
	                               const int st[2], const int st_dx[2], const int st_dy[2], bool persp_overflow,
	                               bool tex_lod_en, bool sharpen, bool detail)
	{
		bool magnify = false, distant = false;
		uint32_t tile_offset = 0;
		if (persp_overflow)
		{
			distant = true;
			lod_frac = 0xff;
		}
		else
		{
			int dx[2], dy[2];
			for (int i = 0; i < 2; i++)
			{
				dx[i] = st_dx[i] - st[i];
				dx[i] ^= dx[i] >> 31;
				dy[i] = st_dy[i] - st[i];
				dy[i] ^= dy[i] >> 31;
			}
			int max_d = std::max(std::max(dx[0], dy[0]), std::max(dx[1], dy[1]));
			if (max_d >= 0x4000)
			{
				distant = true;
				lod_frac = 0xff;
				tile_offset = max_level;
			}
			else if (max_d < 32)
			{
				distant = max_level == 0u;
				magnify = true;
				if (!sharpen && !detail) lod_frac = distant ? 0xff : 0;
				else lod_frac = (std::max(min_lod, max_d) << 3) + (sharpen ? -0x100 : 0);
			}
			else
			{
				int mip_base = std::max(find_msb(max_d >> 5), 0);
				distant = uint32_t(mip_base) >= max_level;
				if (distant && !sharpen && !detail) lod_frac = 0xff;
				else
				{
					lod_frac = ((max_d << 3) >> mip_base) & 0xff;
					tile_offset = uint32_t(mip_base);
				}
			}
		}
		if (tex_lod_en)
		{
			if (distant) tile_offset = max_level;
			if (!detail)
			{
				tile0 = (tile0 + tile_offset) & 7u;
				if (distant || (!sharpen && magnify)) tile1 = tile0;
				else tile1 = (tile0 + 1) & 7u;
			}
			else
			{
				tile1 = (tile0 + tile_offset + ((distant || magnify) ? 1 : 2)) & 7u;
				tile0 = (tile0 + tile_offset + (magnify ? 0 : 1)) & 7u;
			}
		}
	}

	// ======================================================================= combiner
	struct CombIn
	{
		const int *c_muladd, *c_mulsub, *c_mul, *c_add;
		int shade[4];
		int combined[4];
		int texel0[4];
		int texel1[4];
		int lod_frac;
		int noise;
	};

	static int special_expand(int v) { return bfe_s(v - 0x80, 9) + 0x80; }

	static void sel(const CombIn &in, const int rgb_sel[4], const int a_sel[4], int out[4][4])
	{
		// out[k][c]: k = muladd, mulsub, mul, add
		for (int c = 0; c < 3; c++)
		{
			switch (rgb_sel[0])
			{
			case 0: out[0][c] = in.combined[c]; break;
			case 1: out[0][c] = in.texel0[c]; break;
			case 2: out[0][c] = in.texel1[c]; break;
			case 4: out[0][c] = in.shade[c]; break;
			case 7: out[0][c] = in.noise; break;
			case 6: out[0][c] = 0x100; break;
			default: out[0][c] = in.c_muladd[c]; break;
			}
			switch (rgb_sel[1])
			{
			case 0: out[1][c] = in.combined[c]; break;
			case 1: out[1][c] = in.texel0[c]; break;
			case 2: out[1][c] = in.texel1[c]; break;
			case 4: out[1][c] = in.shade[c]; break;
			case 7: out[1][c] = (in.c_mulsub[1] << 8) | in.c_mulsub[2]; break;
			default: out[1][c] = in.c_mulsub[c]; break;
			}
			switch (rgb_sel[2])
			{
			case 0: out[2][c] = in.combined[c]; break;
			case 7: out[2][c] = in.combined[3]; break;
			case 1: out[2][c] = in.texel0[c]; break;
			case 2: out[2][c] = in.texel1[c]; break;
			case 4: out[2][c] = in.shade[c]; break;
			case 8: out[2][c] = in.texel0[3]; break;
			case 9: out[2][c] = in.texel1[3]; break;
			case 11: out[2][c] = in.shade[3]; break;
			case 13: out[2][c] = in.lod_frac; break;
			case 15: out[2][c] = (in.c_mul[1] << 8) | in.c_mul[2]; break;
			default: out[2][c] = in.c_mul[c]; break;
			}
			switch (rgb_sel[3])
			{
			case 0: out[3][c] = in.combined[c]; break;
			case 1: out[3][c] = in.texel0[c]; break;
			case 2: out[3][c] = in.texel1[c]; break;
			case 4: out[3][c] = in.shade[c]; break;
			case 6: out[3][c] = 0x100; break;
			default: out[3][c] = in.c_add[c]; break;
			}
		}
		auto addsub = [&](int s, const int *cst) -> int {
			switch (s)
			{
			case 0: return in.combined[3];
			case 1: return in.texel0[3];
			case 2: return in.texel1[3];
			case 4: return in.shade[3];
			case 6: return 0x100;
			default: return cst[3];
			}
		};
		out[0][3] = addsub(a_sel[0], in.c_muladd);
		out[1][3] = addsub(a_sel[1], in.c_mulsub);
		switch (a_sel[2])
		{
		case 0: out[2][3] = in.lod_frac; break;
		case 1: out[2][3] = in.texel0[3]; break;
		case 2: out[2][3] = in.texel1[3]; break;
		case 4: out[2][3] = in.shade[3]; break;
		default: out[2][3] = in.c_mul[3]; break;
		}
		out[3][3] = addsub(a_sel[3], in.c_add);
	}

	static void combiner_equation(const int v[4][4], int out[4])
	{
		for (int c = 0; c < 4; c++)
		{
			int a = special_expand(v[0][c]);
			int b = special_expand(v[1][c]);
			int cc = bfe_s(v[2][c], 9);
			int d = special_expand(v[3][c]);
			int col = (a - b) * cc;
			col += 0x80;
			out[c] = (col >> 8) + d;
		}
	}

	static void combiner_cycle0(const CombIn &in, const int rgb_sel[4], const int a_sel[4], int alpha_dith,
	                            int coverage, bool cvg_times_alpha, bool alpha_cvg_select, bool alpha_test,
	                            int out[4], int &alpha_ref)
	{
		int v[4][4];
		sel(in, rgb_sel, a_sel, v);
		combiner_equation(v, out);
		if (alpha_test)
		{
			int ca = clampi(bfe_s(out[3] - 0x80, 9) + 0x80, 0, 0xff);
			int ea = ca + ((ca + 1) >> 8);
			if (alpha_cvg_select)
			{
				int m = cvg_times_alpha ? ((ea * coverage + 4) >> 3) : (coverage << 5);
				ea = m;
			}
			else
				ea += alpha_dith;
			alpha_ref = clampi(ea, 0, 0xff);
		}
		else
			alpha_ref = 0;
	}

	static void combiner_cycle1(const CombIn &in, const int rgb_sel[4], const int a_sel[4], int alpha_dith,
	                            int &coverage, bool cvg_times_alpha, bool alpha_cvg_select, int out[4])
	{
		int v[4][4];
		sel(in, rgb_sel, a_sel, v);
		combiner_equation(v, out);
		for (int c = 0; c < 4; c++) out[c] = clamp_9bit_notrunc(out[c]);
		int ea = out[3] + ((out[3] + 1) >> 8);
		int m;
		if (cvg_times_alpha)
		{
			m = (ea * coverage + 4) >> 3;
			coverage = m >> 5;
		}
		else
			m = coverage << 5;
		if (alpha_cvg_select) ea = m;
		else ea += alpha_dith;
		out[3] = clampi(ea, 0, 0xff);
	}

	// ======================================================================= per-primitive record
	struct Prim
	{
		TriSetup setup;
		Attr attr;
		Derived derived;
		Scissor scissor;
		StaticState st;   // normalized
		DepthBlend db;
		TileInfo tiles[8];
		const uint16_t *tmem;
		uint32_t prim_index; // global index used for noise
		int span_ylo, span_yhi;
	};

	struct Shaded
	{
		int combined[4];
		int z_dith;
		int coverage_count;
		int shade_alpha;
	};

	// Span rows of the primitive being rendered, each set up once (span_setup.comp runs one
	// invocation per scanline of a primitive, shading.h reads the rows; rdp_renderer.cpp:1523-1554).
	// Rows span_ylo .. span_yhi + 1 (the last for the pipelined texel1 peek at the next line).
	std::vector<Span> span_rows;
	std::vector<uint8_t> span_row_ready;
	void begin_span_rows(const Prim &p)
	{
		size_t n = p.span_yhi >= p.span_ylo ? size_t(p.span_yhi - p.span_ylo) + 2 : 0;
		if (span_rows.size() < n) span_rows.resize(n);
		span_row_ready.assign(n, 0);
	}
	const Span &span_row(const Prim &p, int y)
	{
		size_t i = size_t(y - p.span_ylo);
		if (!span_row_ready[i])
		{
			span_rows[i] = span_setup(p.setup, p.attr, p.scissor, y);
			span_row_ready[i] = 1;
		}
		return span_rows[i];
	}

	// Scaled span rows of the primitive being rendered upscaled: row r is scanline S * span_ylo + r
	// (the last one is the pipelined texel1 peek at the next line).
	const Span *up_rows = nullptr;
	const Span &scaled_row(const Prim &p, int y, int L) const { return up_rows[y - (p.span_ylo << L)]; }

	// shading.h:38-359; L is log2 of the upscaling factor (0 at 1x), x and y are scaled coordinates.
	bool shade_pixel(const Prim &p, int x, int y, Shaded &out, int fb_size, int dx_mask, int dx_shift, int L = 0)
	{
		const int S = 1 << L;
		if (y < S * p.span_ylo || y > p.span_yhi * S + (S - 1)) return false;
		if (S > 1 && (p.setup.flags & TRI_DISABLE_UPSCALING))
		{
			x &= ~(S - 1);
			y &= ~(S - 1);
		}
		const Span &sp = L ? scaled_row(p, y, L) : span_row(p, y);
		if (!sp.valid) return false;
		const StaticState &st = p.st;
		uint32_t f = st.flags;
		bool tlut = (f & R_TLUT) != 0, tlut_type = (f & R_TLUT_TYPE) != 0, sample_quad = (f & R_SAMPLE_QUAD) != 0;
		bool cvg_times_alpha = (f & R_CVG_TIMES_ALPHA) != 0, alpha_cvg_select = (f & R_ALPHA_CVG_SELECT) != 0;
		bool perspective = (f & R_PERSPECTIVE) != 0, tex_lod_en = (f & R_TEX_LOD) != 0;
		bool sharpen = (f & R_SHARPEN) != 0, detail = (f & R_DETAIL) != 0, aa_enable = (f & R_AA) != 0;
		bool multi_cycle = (f & R_MULTI_CYCLE) != 0, interlace_en = (f & R_INTERLACE_FIELD) != 0;
		bool fill_en = (f & R_FILL) != 0, copy_en = (f & R_COPY) != 0, alpha_test = (f & R_ALPHA_TEST) != 0;
		bool alpha_test_dither = (f & R_ALPHA_TEST_DITHER) != 0, mid_texel = (f & R_MID_TEXEL) != 0;
		bool uses_texel0 = (f & R_USES_TEXEL0) != 0, uses_texel1 = (f & R_USES_TEXEL1) != 0;
		bool uses_pipelined_texel1 = (f & R_USES_PIPELINED_TEXEL1) != 0, uses_lod = (f & R_USES_LOD) != 0;
		bool convert_one = (f & R_CONVERT_ONE) != 0, bilerp0 = (f & R_BILERP0) != 0, bilerp1 = (f & R_BILERP1) != 0;

		if (f & R_NEED_NOISE) reseed_noise(uint32_t(x), uint32_t(y), p.prim_index);
		bool flip = (p.setup.flags & TRI_FLIP) != 0;

		if (copy_en)
		{
			if (!(x >= sp.start_x && x <= sp.end_x)) return false;
			int st2[2], s_offset;
			interpolate_st_copy(sp, p.attr.dstzw_dx, x, perspective, flip, dx_mask, dx_shift, st2, s_offset, L);
			uint32_t tile0 = p.setup.tile & 7u;
			int texel0 = sample_texture_copy(p.tmem, p.tiles[tile0], st2[0], st2[1], s_offset, tlut, fb_size);
			out.z_dith = texel0;
			out.coverage_count = 0x20;
			if (alpha_test && fb_size == 2 && (texel0 & 1) == 0) return false;
			return true;
		}
		else if (fill_en)
		{
			out.coverage_count = 0x40;
			return x >= sp.start_x && x <= sp.end_x;
		}

		int coverage = compute_coverage(sp.xleft, sp.xright, x);
		if (coverage == 0) return false;
		int coverage_count = popc(uint32_t(coverage));
		if (!aa_enable && (coverage & 1) == 0) return false;

		const Derived &d = p.derived;
		int dx = x - sp.base_x;
		int interp_dir = flip ? 1 : -1;
		int shade[4];
		interpolate_rgba(sp.rgba, p.attr.drgba_dx, p.attr.drgba_dy, dx, coverage, shade, L);

		int st2[2] = {}, st_dx[2] = {}, st_dy[2] = {}, z = 0;
		bool persp_overflow = false;
		int tex_dir = interp_dir;
		if (S > 1 && uses_lod && (p.setup.flags & TRI_NATIVE_LOD)) tex_dir *= S;
		interpolate_stz(sp.stzw, p.attr.dstzw_dx, p.attr.dstzw_dy, dx, coverage, perspective, uses_lod, tex_dir,
		                st2, st_dx, st_dy, z, persp_overflow, L);

		uint32_t tile0 = p.setup.tile & 7u;
		uint32_t tile1 = (tile0 + 1) & 7u;
		uint32_t max_level = p.setup.tile >> 3;
		int lod_frac = 0;
		if (uses_lod)
			compute_lod_2cycle(tile0, tile1, lod_frac, max_level, d.min_lod, st2, st_dx, st_dy, persp_overflow,
			                   tex_lod_en, sharpen, detail);

		T4 texel0 = {}, texel1 = {};
		if (uses_texel0)
			texel0 = sample_texture(p.tmem, p.tiles[tile0], st2[0], st2[1], tlut, tlut_type, sample_quad, mid_texel,
			                        false, bilerp0, d.factors, T4{});

		if (uses_pipelined_texel1)
		{
			const Span &next = L ? scaled_row(p, y + 1, L) : span_row(p, y + 1);
			bool valid_line = next.valid;
			bool long_span = sp.lodlength >= 8;
			bool end_span = x == (flip ? sp.end_x : sp.start_x);
			if (end_span && long_span && valid_line)
			{
				int stw[3] = { next.stzw[0] >> 16, next.stzw[1] >> 16, next.stzw[3] >> 16 };
				bool ov = false;
				st_divide(stw, perspective, st2, ov);
			}
			else
				interpolate_st_single(sp.stzw, p.attr.dstzw_dx, dx + interp_dir * S, perspective, st2, L);
			tile1 = tile0;
			uses_texel1 = true;
		}

		if (uses_texel1)
		{
			if (convert_one && !bilerp1)
				texel1 = texture_convert_factors(texel0, d.factors);
			else
				texel1 = sample_texture(p.tmem, p.tiles[tile1], st2[0], st2[1], tlut, tlut_type, sample_quad,
				                        mid_texel, convert_one, bilerp1, d.factors, texel0);
		}

		int rgb_dith, alpha_dith;
		dither_coefficients(x, y >> int(interlace_en), st.dither >> 2, st.dither & 3, rgb_dith, alpha_dith);

		int combined[4];
		int alpha_reference = 0;
		if (multi_cycle)
		{
			CombIn in;
			in.c_muladd = d.c_muladd[0];
			in.c_mulsub = d.c_mulsub[0];
			in.c_mul = d.c_mul[0];
			in.c_add = d.c_add[0];
			for (int c = 0; c < 4; c++)
			{
				in.shade[c] = shade[c];
				in.combined[c] = 0;
				in.texel0[c] = texel0.v[c];
				in.texel1[c] = texel1.v[c];
			}
			in.lod_frac = lod_frac;
			in.noise = noise_combiner();
			int c0[4];
			combiner_cycle0(in, st.rgb[0], st.alpha[0], alpha_dith, coverage_count, cvg_times_alpha,
			                alpha_cvg_select, alpha_test, c0, alpha_reference);
			for (int c = 0; c < 4; c++)
			{
				in.combined[c] = c0[c];
				int tmp = in.texel0[c];
				in.texel0[c] = in.texel1[c];
				in.texel1[c] = tmp;
			}
			in.c_muladd = d.c_muladd[1];
			in.c_mulsub = d.c_mulsub[1];
			in.c_mul = d.c_mul[1];
			in.c_add = d.c_add[1];
			if (f & R_NEED_NOISE_DUAL)
			{
				reseed_noise(uint32_t(x + 1023), uint32_t(y + 7), p.prim_index + 11);
				in.noise = noise_combiner();
			}
			combiner_cycle1(in, st.rgb[1], st.alpha[1], alpha_dith, coverage_count, cvg_times_alpha,
			                alpha_cvg_select, combined);
		}
		else
		{
			CombIn in;
			in.c_muladd = d.c_muladd[1];
			in.c_mulsub = d.c_mulsub[1];
			in.c_mul = d.c_mul[1];
			in.c_add = d.c_add[1];
			for (int c = 0; c < 4; c++)
			{
				in.shade[c] = shade[c];
				in.combined[c] = 0;
				in.texel0[c] = texel0.v[c];
				in.texel1[c] = texel1.v[c];
			}
			in.lod_frac = lod_frac;
			in.noise = noise_combiner();
			combiner_cycle1(in, st.rgb[1], st.alpha[1], alpha_dith, coverage_count, cvg_times_alpha,
			                alpha_cvg_select, combined);
			alpha_reference = combined[3];
		}

		if (aa_enable && coverage_count == 0) return false;
		if (alpha_test)
		{
			int thr = alpha_test_dither ? noise_blend_threshold() : d.blend[3];
			if (alpha_reference < thr) return false;
		}

		for (int c = 0; c < 4; c++) out.combined[c] = combined[c] & 0xff;
		out.z_dith = (z << 9) | rgb_dith;
		out.coverage_count = coverage_count;
		out.shade_alpha = std::min(shade[3] + alpha_dith, 0xff);
		return true;
	}

	// ======================================================================= memory interfacing
	using PixelState = PixelStateSlot;
	uint32_t pass_stamp = 1;

	void load_color(PixelState &ps, uint32_t index) const
	{
		switch (fb.fmt)
		{
		case FB_I4:
		case FB_I8:
		{
			index &= rdram_size - 1;
			int w = vram8(index ^ 3u);
			ps.color[0] = ps.color[1] = ps.color[2] = w;
			ps.color[3] = hid(index >> 1);
			break;
		}
		case FB_RGBA5551:
		{
			index &= (rdram_size >> 1) - 1;
			uint32_t w = vram16(index ^ 1u);
			ps.color[0] = int((w >> 8) & 0xf8u);
			ps.color[1] = int((w >> 3) & 0xf8u);
			ps.color[2] = int((w << 2) & 0xf8u);
			ps.color[3] = ((hid(index) << 5) | int((w & 1) << 7)) & 0xff;
			break;
		}
		case FB_IA88:
		{
			index &= (rdram_size >> 1) - 1;
			uint32_t w = vram16(index ^ 1u);
			ps.color[0] = ps.color[1] = ps.color[2] = int((w >> 8) & 0xff);
			ps.color[3] = int(w & 0xff);
			break;
		}
		default:
		{
			index &= (rdram_size >> 2) - 1;
			uint32_t w = vram32(index);
			for (int c = 0; c < 4; c++) ps.color[c] = int((w >> (24 - 8 * c)) & 0xff);
			break;
		}
		}
	}

	void load_depth(PixelState &ps, uint32_t index) const
	{
		index &= (rdram_size >> 1) - 1;
		uint32_t w = vram16(index ^ 1u);
		ps.depth = int(w >> 2);
		ps.dz = (hid(index) | int((w & 3) << 2)) & 0xff;
	}

	void alias_color_to_depth(PixelState &ps) const
	{
		switch (fb.fmt)
		{
		case FB_RGBA5551:
		{
			ps.dz = ((ps.color[3] >> 3) | (ps.color[2] & 8)) & 0xff;
			uint32_t w = (uint32_t(ps.color[0]) & 0xf8u) << 6;
			w |= (uint32_t(ps.color[1]) & 0xf8u) << 1;
			w |= (uint32_t(ps.color[2]) & 0xf8u) >> 4;
			ps.depth = int(w & 0xffff);
			break;
		}
		case FB_IA88:
		{
			uint32_t w = (uint32_t(ps.color[0]) << 8) | uint32_t(ps.color[3]);
			uint32_t hw = (w & 1u) * 3u;
			ps.depth = int((w >> 2) & 0xffff);
			ps.dz = int((((w & 3u) << 2) | hw) & 0xff);
			break;
		}
		default:
			break;
		}
	}

	void alias_depth_to_color(PixelState &ps) const
	{
		uint32_t w = (uint32_t(ps.depth) << 4) | uint32_t(ps.dz);
		switch (fb.fmt)
		{
		case FB_RGBA5551:
			ps.color[0] = int((w >> 10) & 0xf8u);
			ps.color[1] = int((w >> 5) & 0xf8u);
			ps.color[2] = int(w & 0xf8u);
			ps.color[3] = int((w & 7u) << 5);
			break;
		case FB_IA88:
			ps.color[0] = int((w >> 10) & 0xffu);
			ps.color[3] = int((w >> 2) & 0xffu);
			break;
		default:
			break;
		}
		ps.color_dirty = true;
	}

	void store_color(const PixelState &ps, uint32_t index)
	{
		if (!ps.color_dirty) return;
		switch (fb.fmt)
		{
		case FB_I4:
			index &= rdram_size - 1;
			w_vram8(index ^ 3u, 0);
			if (index & 1u) w_hid(index >> 1, uint8_t(ps.color[3]));
			break;
		case FB_I8:
		{
			index &= rdram_size - 1;
			uint32_t col = (index & 1) ? uint32_t(ps.color[1]) : uint32_t(ps.color[0]);
			w_vram8(index ^ 3u, uint8_t(col));
			if (index & 1u) w_hid(index >> 1, uint8_t((col & 1) * 3));
			break;
		}
		case FB_RGBA5551:
		{
			index &= (rdram_size >> 1) - 1;
			uint32_t r = uint32_t(ps.color[0]) & 0xf8u, g = uint32_t(ps.color[1]) & 0xf8u,
			         b = uint32_t(ps.color[2]) & 0xf8u;
			uint32_t cov = uint32_t(ps.color[3]) >> 5;
			uint32_t w = (r << 8) | (g << 3) | (b >> 2) | (cov >> 2);
			w_vram16(index ^ 1u, uint16_t(w));
			w_hid(index, uint8_t(cov & 3u));
			break;
		}
		case FB_IA88:
		{
			index &= (rdram_size >> 1) - 1;
			uint32_t w = (uint32_t(ps.color[0]) << 8) | uint32_t(ps.color[3]);
			w_vram16(index ^ 1u, uint16_t(w));
			w_hid(index, uint8_t((ps.color[3] & 1) * 3));
			break;
		}
		default:
		{
			index &= (rdram_size >> 2) - 1;
			uint32_t w = (uint32_t(ps.color[0]) << 24) | (uint32_t(ps.color[1]) << 16) | (uint32_t(ps.color[2]) << 8) |
			             uint32_t(ps.color[3]);
			w_vram32(index, w);
			w_hid(2u * index, uint8_t((ps.color[1] & 1) * 3));
			w_hid(2u * index + 1u, uint8_t((ps.color[3] & 1) * 3));
			break;
		}
		}
	}

	void store_depth(const PixelState &ps, uint32_t index, bool alias)
	{
		if (alias || !ps.depth_dirty) return;
		index &= (rdram_size >> 1) - 1;
		w_vram16(index ^ 1u, uint16_t((ps.depth << 2) | (ps.dz >> 2)));
		w_hid(index, uint8_t(ps.dz & 3));
	}

	void decode_memory_color(const PixelState &ps, bool image_read_en, int out[4]) const
	{
		int mc = image_read_en ? (ps.color[3] & 0xe0) : 0xe0;
		switch (fb.fmt)
		{
		case FB_I4: out[0] = out[1] = out[2] = 0; mc = 0xe0; break;
		case FB_I8: out[0] = out[1] = out[2] = ps.color[0]; mc = 0xe0; break;
		case FB_RGBA5551: for (int c = 0; c < 3; c++) out[c] = ps.color[c] & 0xf8; break;
		case FB_IA88: out[0] = out[1] = out[2] = ps.color[0]; break;
		default: for (int c = 0; c < 3; c++) out[c] = ps.color[c]; break;
		}
		out[3] = mc;
	}

	void write_color(PixelState &ps, const int col[4]) const
	{
		if (fb.fmt == FB_I4)
			for (int c = 0; c < 3; c++) ps.color[c] = col[c];
		else
			for (int c = 0; c < 4; c++) ps.color[c] = col[c];
		ps.color_dirty = true;
	}

	void copy_pipeline(PixelState &ps, uint32_t word, bool alias) const
	{
		switch (fb.fmt)
		{
		case FB_I4:
			for (int c = 0; c < 4; c++) ps.color[c] = 0;
			ps.color_dirty = true;
			break;
		case FB_I8:
		{
			int v = int(word & 0xffu);
			int col[4] = { v, v, v, v };
			write_color(ps, col);
			break;
		}
		case FB_RGBA5551:
		{
			int col[4] = { int((word >> 8) & 0xf8u), int((word >> 3) & 0xf8u), int((word << 2) & 0xf8u),
			               int((word & 1) * 0xe0u) };
			write_color(ps, col);
			break;
		}
		default:
			break;
		}
		if (alias) alias_color_to_depth(ps);
	}

	void fill_color_op(PixelState &ps, uint32_t col, bool alias) const
	{
		switch (fb.fmt)
		{
		case FB_RGBA8888:
		{
			int c4[4] = { int((col >> 24) & 0xff), int((col >> 16) & 0xff), int((col >> 8) & 0xff), int(col & 0xff) };
			write_color(ps, c4);
			break;
		}
		case FB_RGBA5551:
		{
			col >>= ((ps.color_index & 1u) ^ 1u) * 16u;
			int c4[4] = { int((col >> 8) & 0xf8u), int((col >> 3) & 0xf8u), int((col << 2) & 0xf8u),
			              int((col & 1u) * 0xe0u) };
			write_color(ps, c4);
			break;
		}
		case FB_IA88:
		{
			col >>= ((ps.color_index & 1u) ^ 1u) * 16u;
			col &= 0xffffu;
			int r = int((col >> 8) & 0xff), a = int(col & 0xff);
			int c4[4] = { r, r, r, a };
			write_color(ps, c4);
			break;
		}
		case FB_I8:
		{
			col >>= ((ps.color_index & 3u) ^ 3u) * 8u;
			col &= 0xffu;
			int c4[4] = { int(col), int(col), int(col), int(col) };
			write_color(ps, c4);
			break;
		}
		default:
			break;
		}
		if (alias) alias_color_to_depth(ps);
	}

	// depth_test.h:41-144
	static bool depth_test(int z, int dz, int dz_compressed, int cur_depth, int cur_dz, int &coverage_count,
	                       int cur_cov, bool z_compare, int z_mode, bool force_blend, bool aa_enable, bool &blend_en,
	                       bool &coverage_wrap, int blend_shift[2])
	{
		bool pass;
		if (z_compare)
		{
			int memory_z = z_decompress(cur_depth);
			int memory_dz = 1 << cur_dz;
			int precision_factor = (cur_depth >> 11) & 0xf;
			bool coplanar = false;
			blend_shift[0] = clampi(dz_compressed - cur_dz, 0, 4);
			blend_shift[1] = clampi(cur_dz - dz_compressed, 0, 4);
			if (precision_factor < 3)
			{
				if (memory_dz != 0x8000) memory_dz = std::max(memory_dz << 1, 16 >> precision_factor);
				else
				{
					coplanar = true;
					memory_dz = 0xffff;
				}
			}
			int combined_dz = dz | memory_dz;
			if (combined_dz != 0) combined_dz = 1 << find_msb(combined_dz);
			int combined_dz_i = combined_dz;
			combined_dz <<= 3;
			bool farther = coplanar || ((z + combined_dz) >= memory_z);
			bool overflow = (coverage_count + cur_cov) >= 8;
			blend_en = force_blend || (!overflow && aa_enable && farther);
			coverage_wrap = overflow;
			pass = false;
			bool max_z = memory_z == 0x3ffff;
			bool front = z < memory_z;
			int z_closest = z - combined_dz;
			bool nearer = coplanar || (z_closest <= memory_z);
			switch (z_mode)
			{
			case 0:
				pass = max_z || (overflow ? front : nearer);
				break;
			case 1:
				if (!front || !farther || !overflow)
					pass = max_z || (overflow ? front : nearer);
				else
				{
					combined_dz_i = std::max(find_msb(combined_dz_i & 0xffff), 0);
					int cvg_coeff = ((memory_z >> combined_dz_i) - (z >> combined_dz_i)) & 0xf;
					coverage_count = std::min((cvg_coeff * coverage_count) >> 3, 8);
					pass = true;
				}
				break;
			case 2:
				pass = front || max_z;
				break;
			default:
				pass = farther && nearer && !max_z;
				break;
			}
		}
		else
		{
			blend_shift[0] = 0;
			blend_shift[1] = std::min(0xf - dz_compressed, 4);
			bool overflow = (coverage_count + cur_cov) >= 8;
			blend_en = force_blend || (!overflow && aa_enable);
			coverage_wrap = overflow;
			pass = true;
		}
		return pass;
	}

	static int z_decompress(int z)
	{
		int exponent = z >> 11;
		int mantissa = z & 0x7ff;
		int shift = std::max(6 - exponent, 0);
		int base = 0x40000 - (0x40000 >> exponent);
		return (mantissa << shift) + base;
	}

	static int z_compress(int z)
	{
		int inv_z = std::max(0x3ffff - z, 1);
		int exponent = 17 - find_msb(inv_z);
		exponent = clampi(exponent, 0, 7);
		int shift = std::max(6 - exponent, 0);
		int mantissa = (z >> shift) & 0x7ff;
		return ((exponent << 11) + mantissa) & 0xffff;
	}

	// blender.h:55-143
	void blender(const int pixel[4], const int memory[4], const int fog[4], const int blendc[4], int shade_alpha,
	             const BlendModes &m, bool force_blend, bool blend_en, bool color_on_cvg, bool coverage_wrap,
	             const int blend_shift[2], bool final_cycle, int out[3]) const
	{
		auto pick = [&](int s) -> const int * {
			switch (s)
			{
			case 0: return pixel;
			case 1: return memory;
			case 2: return blendc;
			default: return fog;
			}
		};
		const int *rgb1 = pick(m.m2a);
		if (final_cycle && color_on_cvg && !coverage_wrap)
		{
			for (int c = 0; c < 3; c++) out[c] = rgb1[c];
			return;
		}
		const int *rgb0 = pick(m.m1a);
		if (final_cycle)
		{
			if (!blend_en || (m.m1b == 0 && m.m2b == 0 && pixel[3] == 0xff))
			{
				for (int c = 0; c < 3; c++) out[c] = rgb0[c];
				return;
			}
		}
		int a0, a1;
		switch (m.m1b)
		{
		case 0: a0 = pixel[3]; break;
		case 1: a0 = fog[3]; break;
		case 2: a0 = shade_alpha; break;
		default: a0 = 0; break;
		}
		switch (m.m2b)
		{
		case 0: a1 = ~a0 & 0xff; break;
		case 1: a1 = memory[3]; break;
		case 2: a1 = 0xff; break;
		default: a1 = 0; break;
		}
		a0 >>= 3;
		a1 >>= 3;
		if (m.m2b == 1)
		{
			a0 = (a0 >> blend_shift[0]) & 0x3c;
			a1 = (a1 >> blend_shift[1]) | 3;
		}
		int bl[3];
		for (int c = 0; c < 3; c++) bl[c] = rgb0[c] * a0 + rgb1[c] * (a1 + 1);
		if (!final_cycle || force_blend)
		{
			for (int c = 0; c < 3; c++) out[c] = (bl[c] >> 5) & 0xff;
		}
		else
		{
			int sum = (a0 >> 2) + (a1 >> 2) + 1;
			for (int c = 0; c < 3; c++)
			{
				int v = (bl[c] >> 2) & 0x7ff;
				out[c] = blender_lut[((sum << 11) | v) & 0x7fff];
			}
		}
	}

	// memory_interfacing.h:488-571
	bool depth_blend_op(PixelState &ps, const Prim &p, const Shaded &sh, bool alias)
	{
		int z = sh.z_dith >> 9;
		int dith = sh.z_dith & 0x1ff;
		int coverage_count = sh.coverage_count;
		const DepthBlend &db = p.db;
		const Derived &d = p.derived;
		bool force_blend = (db.flags & DB_FORCE_BLEND) != 0;
		bool z_compare = (db.flags & DB_DEPTH_TEST) != 0;
		bool z_update = (db.flags & DB_DEPTH_UPDATE) != 0;
		bool image_read = (db.flags & DB_IMAGE_READ) != 0;
		bool color_on_cvg = (db.flags & DB_COLOR_ON_CVG) != 0;
		bool multi = (db.flags & DB_MULTI_CYCLE) != 0;
		bool aa = (db.flags & DB_AA) != 0;
		bool dither_en = (db.flags & DB_DITHER) != 0;

		int memory[4];
		decode_memory_color(ps, image_read, memory);
		int memory_coverage = memory[3] >> 5;
		bool blend_en = false, coverage_wrap = false;
		int blend_shift[2] = { 0, 0 };
		bool z_pass = depth_test(z, d.dz, d.dz_compressed, ps.depth, ps.dz, coverage_count, memory_coverage,
		                         z_compare, db.z_mode, force_blend, aa, blend_en, coverage_wrap, blend_shift);
		if (z_pass && (!aa || coverage_count != 0))
		{
			int pixel[4] = { sh.combined[0], sh.combined[1], sh.combined[2], sh.combined[3] };
			BlendModes m = db.cyc[0];
			if (multi)
			{
				int tmp[3];
				blender(pixel, memory, d.fog, d.blend, sh.shade_alpha, m, force_blend, blend_en, color_on_cvg,
				        coverage_wrap, blend_shift, false, tmp);
				pixel[0] = tmp[0];
				pixel[1] = tmp[1];
				pixel[2] = tmp[2];
				m = db.cyc[1];
			}
			int rgb[3];
			blender(pixel, memory, d.fog, d.blend, sh.shade_alpha, m, force_blend, blend_en, color_on_cvg,
			        coverage_wrap, blend_shift, true, rgb);
			if (dither_en) rgb_dither(rgb, dith);
			int new_cov = blend_coverage(coverage_count, memory_coverage, blend_en, db.coverage_mode);
			int col[4] = { rgb[0], rgb[1], rgb[2], (new_cov << 5) & 0xff };
			write_color(ps, col);
			if (z_update)
			{
				ps.depth = z_compress(z);
				ps.dz = d.dz_compressed;
				ps.depth_dirty = true;
				if (alias) alias_depth_to_color(ps);
			}
			else if (alias)
				alias_color_to_depth(ps);
			return true;
		}
		return false;
	}

	// ======================================================================= draw
	void fixup_triangle_setup(TriSetup &s) const
	{
		int start_y = s.yh & ~3;
		if (s.ym < start_y) s.ym = 0x7fff;
		if (static_state.flags & R_INTERLACE_FIELD)
		{
			s.flags |= TRI_INTERLACE_FIELD;
			if (static_state.flags & R_INTERLACE_KEEP_ODD) s.flags |= TRI_INTERLACE_KEEP_ODD;
		}
		if (static_state.flags & (R_COPY | R_FILL)) s.flags |= TRI_FILL_COPY_RASTER;
	}

	void draw_primitive(TriSetup setup, const Attr &attr_in)
	{
		fixup_triangle_setup(setup);
		Prim p;
		p.setup = setup;
		p.attr = attr_in;
		if (constants.use_prim_depth)
		{
			p.attr.stzw[2] = constants.prim_depth;
			p.attr.dstzw_dx[2] = 0;
			p.attr.dstzw_de[2] = 0;
			p.attr.dstzw_dy[2] = 0;
		}
		p.derived = build_derived(attr_in);
		p.scissor = scissor;
		deduce_static_texture_state();
		deduce_noise_state();
		p.st = normalize_static_state(static_state);
		p.db = depth_blend;
		for (int i = 0; i < 8; i++) p.tiles[i] = tiles[i];
		p.tmem = tmem;
		p.prim_index = primitive_counter++;

		// Span job range (rdp_renderer.cpp:1523-1554).
		int min_sub = std::max(int(setup.yh), scissor.ylo);
		int max_sub = std::min(int(setup.yl) - 1, scissor.yhi - 1);
		ref.prim(raw_other_modes[0], raw_other_modes[1], raw_combine[0], raw_combine[1], (max_sub >> 2) - (min_sub >> 2) + 1);
		int ylo = min_sub >> 2, yhi = max_sub >> 2;
		if (yhi < ylo) { ylo = 0; yhi = -1; }
		p.span_ylo = ylo;
		p.span_yhi = yhi;
		deduced_height = std::max<uint32_t>(deduced_height, uint32_t(std::max((max_sub >> 2) + 1, 0)));
		color_pending = true;
		if (depth_blend.flags & DB_DEPTH_UPDATE) depth_pending = true;
		if (yhi >= ylo) pass_span_prims++;
		if (up_log2 && yhi >= ylo)
		{
			// The upscaled pass renders after the pass ends: keep the primitive with its TMEM.
			if (!tmem_snap) tmem_snap = std::make_shared<std::vector<uint16_t>>(tmem, tmem + 2048);
			pass_list.push_back({ p, tmem_snap });
			pass_list.back().p.tmem = tmem_snap->data();
		}
		if (fb.width != 0 && yhi >= ylo) render_primitive(p);
		if (++pass_prims >= 256) end_pass();
	}

	// Ends the current render pass: stores every pixel touched in it (finish_tile).  With upscaling
	// the pass is also rendered at the scaled resolution (Renderer::flush_queues,
	// rdp_renderer.cpp:2953-2986): the 1x pass is bracketed by the "pre" and "post" updates of the
	// upscaled domain (submit_render_pass, 2223-2285) and followed by the upscaled pass
	// (submit_render_pass_upscaled, 2287-2342); with super-sampled readback only the upscaled pass
	// runs and is resolved into RDRAM.
	void end_pass()
	{
		const bool need_render_pass = fb.width != 0 && deduced_height != 0 && pass_span_prims != 0;
		if (up_log2 && !ssaa && need_render_pass) update_upscaled_domain(false);
		if (!touched.empty())
		{
			bool alias = fb.addr == fb.depth_addr;
			uint32_t depth_index = fb.depth_addr >> 1;
			if (!ssaa)
				for (uint32_t slot : touched)
				{
					const PixelState &ps = pixel_cache[slot];
					uint32_t x = slot & 1023u, y = slot >> 10;
					store_color(ps, ps.color_index);
					store_depth(ps, depth_index + fb.width * y + x, alias);
				}
			touched.clear();
		}
		if (up_log2 && (ssaa || (need_render_pass && render_upscaled_format())))
		{
			if (ssaa)
			{
				update_upscaled_domain(false);
				clear_ssaa_mask();
			}
			else
				update_upscaled_domain(true);
			render_upscaled();
			if (ssaa) ssaa_resolve();
		}
		pass_list.clear();
		pass_span_prims = 0;
		pass_stamp++;
		pass_prims = pass_uploads = 0;
		deduced_height = 0;
		color_pending = depth_pending = false;
	}

	bool upload_needs_flush(uint32_t addr) const
	{
		if (color_pending)
		{
			uint32_t offset = (addr - fb.addr) & (rdram_size - 1);
			uint32_t pixels = deduced_height * fb.width;
			if (fb.fmt == FB_RGBA5551 || fb.fmt == FB_I8) offset >>= 1;
			else if (fb.fmt == FB_RGBA8888) offset >>= 2;
			if (offset < pixels) return true;
		}
		if (depth_pending)
		{
			uint32_t offset = ((addr - fb.depth_addr) & (rdram_size - 1)) >> 1;
			if (offset < deduced_height * fb.width) return true;
		}
		return false;
	}

	void render_primitive(const Prim &p)
	{
		int fb_size, dx_mask, dx_shift;
		uint32_t addr_index;
		switch (fb.fmt)
		{
		case FB_I4: fb_size = 0; dx_mask = 0; dx_shift = 0; addr_index = fb.addr; break;
		case FB_I8: fb_size = 1; dx_mask = ~7; dx_shift = 3; addr_index = fb.addr; break;
		case FB_RGBA5551:
		case FB_IA88: fb_size = 2; dx_mask = ~3; dx_shift = 2; addr_index = fb.addr >> 1; break;
		default: fb_size = 4; dx_mask = ~1; dx_shift = 1; addr_index = fb.addr >> 2; break;
		}
		uint32_t depth_index = fb.depth_addr >> 1;
		bool alias = fb.addr == fb.depth_addr;
		int width = int(fb.width);
		int tiles_x = (width + 7) / 8;
		int ty0 = p.span_ylo / 8, ty1 = p.span_yhi / 8;
		begin_span_rows(p);
		for (int ty = ty0; ty <= ty1; ty++)
		{
			for (int tx = 0; tx < tiles_x; tx++)
			{
				int lox = tx * 8, loy = ty * 8;
				int hix = std::min(lox + 7, width - 1), hiy = loy + 7;
				if (!bin_primitive(p.setup, lox, loy, hix, hiy, p.scissor)) continue;
				for (int y = loy; y <= hiy; y++)
				{
					for (int x = lox; x <= hix; x++)
					{
						Shaded sh = {};
						if (!shade_pixel(p, x, y, sh, fb_size, dx_mask, dx_shift)) continue;
						uint32_t ci = addr_index + uint32_t(width) * uint32_t(y) + uint32_t(x);
						uint32_t di = depth_index + uint32_t(width) * uint32_t(y) + uint32_t(x);
						uint32_t slot = uint32_t(y) * 1024u + uint32_t(x);
						PixelState &ps = pixel_cache[slot];
						if (ps.pass_stamp != pass_stamp)
						{
							ps = {};
							ps.pass_stamp = pass_stamp;
							ps.color_index = ci;
							load_color(ps, ci);
							load_depth(ps, di);
							touched.push_back(slot);
						}
						// A fragment is a pixel write by this primitive (colour and/or depth).
						bool wrote;
						if (sh.coverage_count & 0x40)
						{
							fill_color_op(ps, p.derived.fill_color, alias);
							wrote = fb.fmt != FB_I4;
						}
						else if (sh.coverage_count & 0x20)
						{
							copy_pipeline(ps, uint32_t(sh.z_dith), alias);
							wrote = fb.fmt == FB_I4 || fb.fmt == FB_I8 || fb.fmt == FB_RGBA5551;
						}
						else
							wrote = depth_blend_op(ps, p, sh, alias);
						if (wrote) fragments++;
					}
				}
			}
		}
	}

	// ======================================================================= upscaling
	// Internal upscaling by S = 2, 4 or 8 (Renderer::init_internal_upscaling_factor,
	// rdp_renderer.cpp:545-601).  The multisampled copy of RDRAM holds S * S slices of RDRAM (and of
	// hidden RDRAM, initialised to 3): pixel (x, y) of the scaled image lives in slice
	// (y % S) * S + x % S, at the address of native pixel (x / S, y / S) (memory_interfacing.h:
	// 286-362).  A reference copy of RDRAM (initially zero) records what the multisampled copy
	// already reflects.
	int up_log2 = 0;
	bool ssaa = false, ssaa_dither = false;
	std::vector<uint8_t> ms_rdram, ms_hidden, up_reference;
	std::vector<uint32_t> ssaa_mask; // 2 bits (colour, depth written) per native pixel, 4x4 pixels a word
	struct PassPrim
	{
		Prim p;
		std::shared_ptr<std::vector<uint16_t>> tmem;
	};
	std::vector<PassPrim> pass_list;                  // the pass's primitives with span rows
	std::shared_ptr<std::vector<uint16_t>> tmem_snap; // TMEM as drawn primitives see it since the last upload

	bool set_upscaling(int factor, bool super_sampled, bool dither)
	{
		int l = factor == 2 ? 1 : factor == 4 ? 2 : factor == 8 ? 3 : factor == 1 ? 0 : -1;
		if (l < 0 || hidden_size != rdram_size / 2) return false;
		end_pass();
		up_log2 = l;
		ssaa = l && super_sampled;
		ssaa_dither = ssaa && dither;
		const size_t n = size_t(1) << (2 * l);
		ms_rdram.assign(l ? n * rdram_size : 0, 0);
		ms_hidden.assign(l ? n * hidden_size : 0, 0x03);
		up_reference.assign(l ? rdram_size : 0, 0);
		ssaa_mask.assign(ssaa ? (1024 / 4) * (1024 / 4) : 0, 0);
		return true;
	}

	// Renderer::should_render_upscaled (rdp_renderer.cpp:2997-3009): 16/32-bit images at least
	// 256 pixels wide.
	bool render_upscaled_format() const
	{
		return (fb.fmt == FB_RGBA5551 || fb.fmt == FB_RGBA8888) && fb.width >= 256;
	}
	static int pixel_size_log2(int fmt)
	{
		return fmt == FB_RGBA8888 ? 2 : (fmt == FB_RGBA5551 || fmt == FB_IA88) ? 1 : 0;
	}

	// One element of update_upscaled_domain_pre.comp (post = false: RDRAM bytes that differ from the
	// reference copy are written to every sample, with their hidden bits, and recorded) or of
	// update_upscaled_domain_post.comp (post = true: the reference copy takes RDRAM).
	void upscale_element(uint32_t index, int psl2, bool post)
	{
		const uint32_t n = 1u << (2 * up_log2), hs = rdram_size >> 1;
		index &= (rdram_size >> psl2) - 1;
		const uint32_t b = index << psl2, bytes = 1u << psl2;
		if (post)
		{
			memcpy(&up_reference[b], &rdram[b], bytes);
			return;
		}
		if (!memcmp(&up_reference[b], &rdram[b], bytes)) return;
		for (uint32_t i = 0; i < n; i++)
		{
			memcpy(&ms_rdram[b + size_t(i) * rdram_size], &rdram[b], bytes);
			uint8_t *mh = &ms_hidden[size_t(i) * hs];
			if (psl2 == 0)
			{
				uint32_t m = index ^ 3u;
				if (m & 1u) mh[m >> 1] = hidden[(m >> 1) & (hidden_size - 1)];
			}
			else if (psl2 == 1)
			{
				uint32_t m = index ^ 1u;
				mh[m] = hidden[m & (hidden_size - 1)];
			}
			else
			{
				mh[2 * index] = hidden[(2 * index) & (hidden_size - 1)];
				mh[2 * index + 1] = hidden[(2 * index + 1) & (hidden_size - 1)];
			}
		}
		memcpy(&up_reference[b], &rdram[b], bytes);
	}

	// Renderer::submit_update_upscaled_domain (rdp_renderer.cpp:1943-2035): `pixels` elements of the
	// image at `addr` (word aligned, whole words) and of the depth image at `depth_addr` unless the
	// two coincide.
	void upscale_range(uint32_t addr, uint32_t depth_addr, uint32_t pixels, int psl2, bool post)
	{
		addr &= ~3u;
		depth_addr &= ~3u;
		const uint32_t align = 4u >> psl2;
		pixels = (pixels + align - 1) & ~(align - 1);
		const bool alias = addr == depth_addr;
		for (uint32_t i = 0; i < pixels; i++)
		{
			upscale_element((addr >> psl2) + i, psl2, post);
			if (!alias) upscale_element((depth_addr >> 1) + i, 1, post);
		}
	}
	void update_upscaled_domain(bool post)
	{
		upscale_range(fb.addr, fb.depth_addr, fb.width * deduced_height, pixel_size_log2(fb.fmt), post);
	}

	// clear_super_sampled_write_mask.comp over the image's 4x4 blocks (rdp_renderer.cpp:2037-2060).
	void clear_ssaa_mask()
	{
		const uint32_t words = ((fb.width + 3) / 4) * ((deduced_height + 3) / 4);
		std::fill(ssaa_mask.begin(), ssaa_mask.begin() + std::min<size_t>(words, ssaa_mask.size()), 0u);
	}

	// The pass at the scaled resolution: depth_blend.comp per 8x8 tile of the scaled image, over the
	// pass's primitives in order, with the scaled span rows (span_setup.comp), binning
	// (binning.h) and shading (shading.h).
	void render_upscaled()
	{
		if (!fb.width || !deduced_height || pass_list.empty()) return;
		const int L = up_log2, S = 1 << L;
		int fb_size, dx_mask, dx_shift;
		uint32_t addr_index;
		switch (fb.fmt)
		{
		case FB_I4: fb_size = 0; dx_mask = 0; dx_shift = 0; addr_index = fb.addr; break;
		case FB_I8: fb_size = 1; dx_mask = ~7; dx_shift = 3; addr_index = fb.addr; break;
		case FB_RGBA5551:
		case FB_IA88: fb_size = 2; dx_mask = ~3; dx_shift = 2; addr_index = fb.addr >> 1; break;
		default: fb_size = 4; dx_mask = ~1; dx_shift = 1; addr_index = fb.addr >> 2; break;
		}
		const uint32_t depth_index = fb.depth_addr >> 1;
		const bool alias = fb.addr == fb.depth_addr;
		const int width = int(fb.width), ws = width * S, hs = int(deduced_height) * S;

		std::vector<std::vector<Span>> rows(pass_list.size());
		for (size_t k = 0; k < pass_list.size(); k++)
		{
			const Prim &p = pass_list[k].p;
			const int n = (p.span_yhi - p.span_ylo + 1) * S + 1;
			rows[k].resize(size_t(n));
			for (int r = 0; r < n; r++) rows[k][size_t(r)] = span_setup(p.setup, p.attr, p.scissor, S * p.span_ylo + r, L);
		}

		uint8_t *const native_rd = mem_rd, *const native_hd = mem_hd;
		auto select_slice = [&](int x, int y) {
			const uint32_t slice = uint32_t(((y & (S - 1)) << L) + (x & (S - 1)));
			mem_rd = ms_rdram.data() + size_t(slice) * rdram_size;
			mem_hd = ms_hidden.data() + size_t(slice) * (rdram_size >> 1);
		};
		const int tiles_x = (ws + 7) / 8, tiles_y = (hs + 7) / 8;
		PixelState px[64];
		for (int ty = 0; ty < tiles_y; ty++)
			for (int tx = 0; tx < tiles_x; tx++)
			{
				const int lox = tx * 8, loy = ty * 8, hix = std::min(lox + 7, ws - 1), hiy = std::min(loy + 7, hs - 1);
				for (int y = loy; y <= hiy; y++)
					for (int x = lox; x <= hix; x++)
					{
						PixelState &ps = px[(y - loy) * 8 + (x - lox)];
						ps = {};
						const uint32_t off = uint32_t(width) * uint32_t(y >> L) + uint32_t(x >> L);
						ps.color_index = addr_index + off; // the fill colour's half / byte follows it
						select_slice(x, y);
						load_color(ps, addr_index + off);
						load_depth(ps, depth_index + off);
					}
				for (size_t k = 0; k < pass_list.size(); k++)
				{
					const Prim &p = pass_list[k].p;
					if (!bin_primitive(p.setup, lox, loy, hix, hiy, p.scissor, S)) continue;
					up_rows = rows[k].data();
					for (int y = loy; y <= hiy; y++)
						for (int x = lox; x <= hix; x++)
						{
							Shaded sh = {};
							if (!shade_pixel(p, x, y, sh, fb_size, dx_mask, dx_shift, L)) continue;
							PixelState &ps = px[(y - loy) * 8 + (x - lox)];
							if (sh.coverage_count & 0x40) fill_color_op(ps, p.derived.fill_color, alias);
							else if (sh.coverage_count & 0x20) copy_pipeline(ps, uint32_t(sh.z_dith), alias);
							else depth_blend_op(ps, p, sh, alias);
						}
				}
				up_rows = nullptr;
				for (int y = loy; y <= hiy; y++)
					for (int x = lox; x <= hix; x++)
					{
						const PixelState &ps = px[(y - loy) * 8 + (x - lox)];
						const uint32_t xn = uint32_t(x >> L), yn = uint32_t(y >> L);
						const uint32_t off = uint32_t(width) * yn + xn;
						select_slice(x, y);
						store_color(ps, addr_index + off);
						store_depth(ps, depth_index + off, alias);
						if (ssaa)
						{
							// emit_scaled_write_masks (memory_interfacing.h:305-337).
							const uint32_t block = (yn >> 2) * ((uint32_t(width) + 3) >> 2) + (xn >> 2);
							const uint32_t word = (uint32_t(ps.color_dirty) + 2u * uint32_t(ps.depth_dirty))
							                      << (2 * ((xn & 3) + (yn & 3) * 4));
							if (block < ssaa_mask.size()) ssaa_mask[block] |= word;
						}
					}
			}
		mem_rd = native_rd;
		mem_hd = native_hd;
	}

	// update_upscaled_domain_resolve.comp: every native pixel of the image that a sample wrote takes
	// the average of its samples (colour; RGBA5551 with an optional ordered dither) or its first
	// sample (depth), in RDRAM and in the reference copy.  Hidden RDRAM is not written.
	void ssaa_resolve()
	{
		static const uint32_t bayer[16] = { 0, 4, 1, 5, 4, 0, 5, 1, 3, 7, 2, 6, 7, 3, 6, 2 };
		const uint32_t n = 1u << (2 * up_log2), w = fb.width, h = deduced_height;
		const int psl2 = pixel_size_log2(fb.fmt);
		const uint32_t color_base = fb.addr >> psl2, depth_base = fb.depth_addr >> 1;
		const bool alias = fb.addr == fb.depth_addr;
		auto rd16 = [](const uint8_t *m, uint32_t i) { return uint32_t(m[2 * i]) | (uint32_t(m[2 * i + 1]) << 8); };
		auto wr16 = [](uint8_t *m, uint32_t i, uint32_t v) { m[2 * i] = uint8_t(v); m[2 * i + 1] = uint8_t(v >> 8); };
		auto rd32 = [](const uint8_t *m, uint32_t i) {
			return uint32_t(m[4 * i]) | (uint32_t(m[4 * i + 1]) << 8) | (uint32_t(m[4 * i + 2]) << 16) |
			       (uint32_t(m[4 * i + 3]) << 24);
		};
		auto wr32 = [](uint8_t *m, uint32_t i, uint32_t v) {
			for (int k = 0; k < 4; k++) m[4 * i + k] = uint8_t(v >> (8 * k));
		};
		for (uint32_t y = 0; y < h; y++)
			for (uint32_t x = 0; x < w; x++)
			{
				const uint32_t index = y * w + x;
				const uint32_t block = (x >> 2) + (y >> 2) * ((w + 3) >> 2);
				const uint32_t wm = block < ssaa_mask.size() ? ssaa_mask[block] >> (2 * ((x & 3) + 4 * (y & 3))) : 0u;
				if (wm & 1u)
				{
					uint32_t ci = color_base + index;
					if (psl2 == 0)
					{
						// The shader sums the first sample NUM_SAMPLES times: the result is that sample.
						ci = (ci & (rdram_size - 1)) ^ 3u;
						rdram[ci] = up_reference[ci] = ms_rdram[ci];
					}
					else if (psl2 == 1)
					{
						ci = (ci & ((rdram_size >> 1) - 1)) ^ 1u;
						uint32_t sum[4] = { 0, 0, 0, 0 };
						for (uint32_t i = 0; i < n; i++)
						{
							uint32_t v = rd16(ms_rdram.data() + size_t(i) * rdram_size, ci);
							sum[0] += (v >> 11) & 0x1f;
							sum[1] += (v >> 6) & 0x1f;
							sum[2] += (v >> 1) & 0x1f;
							sum[3] += v & 1;
						}
						for (int c = 0; c < 4; c++)
						{
							if (ssaa_dither) sum[c] = (8 * sum[c] + bayer[(y & 3) * 4 + (x & 3)] * n) / (8 * n);
							else sum[c] = (sum[c] + (n >> 1)) / n;
						}
						uint32_t enc = (sum[0] << 11) | (sum[1] << 6) | (sum[2] << 1) | sum[3];
						wr16(rdram.data(), ci, enc & 0xffff);
						wr16(up_reference.data(), ci, enc & 0xffff);
					}
					else
					{
						ci &= (rdram_size >> 2) - 1;
						uint32_t sum[4] = { 0, 0, 0, 0 };
						for (uint32_t i = 0; i < n; i++)
						{
							uint32_t v = rd32(ms_rdram.data() + size_t(i) * rdram_size, ci);
							for (int c = 0; c < 4; c++) sum[c] += (v >> (24 - 8 * c)) & 0xff;
						}
						uint32_t enc = 0;
						for (int c = 0; c < 4; c++) enc |= (((sum[c] + (n >> 1)) / n) & 0xffu) << (24 - 8 * c);
						wr32(rdram.data(), ci, enc);
						wr32(up_reference.data(), ci, enc);
					}
				}
				if (!alias && (wm & 2u))
				{
					const uint32_t di = ((depth_base + index) & ((rdram_size >> 1) - 1)) ^ 1u;
					const uint32_t v = rd16(ms_rdram.data(), di);
					wr16(rdram.data(), di, v);
					wr16(up_reference.data(), di, v);
				}
			}
	}

	// ======================================================================= TMEM upload (tmem_update.comp)
	static int compute_upload_t(int offset, float inv_stride)
	{
		volatile float a = float(offset) + 0.5f;
		volatile float b = a * inv_stride;
		return int(b);
	}

	bool update_tmem_32(const UploadInfo &info, int tmem16_index, bool upper, bool yuv, uint32_t &value) const
	{
		int tmem16_offset = (info.tmem_offset & 0x7ff) >> 1;
		int stride = info.tmem_stride_words;
		int pixel_offset = (tmem16_index - tmem16_offset) & 0x3ff;
		int upload_x, upload_y, upload_x_xor = 0;
		if (info.mode == MODE_BLOCK)
		{
			int word_offset = pixel_offset >> 1;
			if (info.tmem_stride_words == 0)
			{
				int f = word_offset & ~1, sdc = f + 1;
				int ft = (f * info.dxt) >> 16, st = (sdc * info.dxt) >> 16;
				if (ft != st)
				{
					int fw = f ^ (ft & 1), sw = sdc ^ (st & 1);
					if (sw == word_offset) upload_x_xor = (st & 1) << 1;
					else if (fw == word_offset) upload_x_xor = (ft & 1) << 1;
					else return false;
				}
				else
					upload_x_xor ^= (ft & 1) << 1;
			}
			else
			{
				int min_t = compute_upload_t(word_offset & ~1, info.min_t_mod);
				int max_t = compute_upload_t(word_offset | 1, info.max_t_mod);
				int max_wc = (word_offset | 1) - stride * min_t;
				int min_wc = (word_offset & ~1) - stride * max_t;
				min_t = std::max(min_t, (min_wc * info.dxt) >> 16);
				max_t = std::min(max_t, (max_wc * info.dxt) >> 16);
				bool found = false;
				for (int t = max_t; t >= min_t; t--)
				{
					int c1 = (word_offset & ~1) - stride * t;
					int c2 = (word_offset | 1) - stride * t;
					int t1 = (c1 * info.dxt) >> 16;
					int t2 = (c2 * info.dxt) >> 16;
					if (((c2 + t2 * stride) ^ (t2 & 1)) == word_offset)
					{
						found = true;
						pixel_offset = (c2 << 1) + (pixel_offset & 1);
						break;
					}
					else if (((c1 + t1 * stride) ^ (t1 & 1)) == word_offset)
					{
						found = true;
						pixel_offset = (c1 << 1) + (pixel_offset & 1);
						break;
					}
				}
				if (!found) return false;
			}
			upload_x = pixel_offset;
			upload_y = 0;
		}
		else if (stride == 0)
		{
			upload_x = pixel_offset;
			upload_y = info.height - 1;
		}
		else
		{
			upload_y = compute_upload_t(pixel_offset, info.inv_tmem_stride_words);
			upload_x = pixel_offset - upload_y * stride;
			if (upload_y >= info.height)
			{
				upload_x += stride * (upload_y - info.height + 1);
				upload_y = info.height - 1;
			}
		}
		int last_line_x = upload_x ^ ((upload_y & 1) << 1);
		if (last_line_x >= info.width && upload_y > 0)
		{
			upload_y--;
			upload_x += stride;
		}
		int iteration_offset = 0;
		upload_x ^= ((upload_y & 1) << 1) | upload_x_xor;
		if (info.vram_size == 3 || yuv)
			iteration_offset = 4 * (upload_x & ~1);
		else if (info.vram_size == 2)
		{
			if (upload_x & 2)
			{
				if (upload_y > 0)
				{
					upload_y--;
					upload_x += stride;
					upload_x ^= 2;
				}
				else
					return false;
			}
			iteration_offset = 2 * (upload_x & ~1);
		}
		else if (info.vram_size == 1)
		{
			for (int i = 0; i < 4 && upload_y > 0 && (upload_x & 6) != 0; i++)
			{
				upload_y--;
				upload_x += stride;
				upload_x ^= 2;
			}
			if (upload_x & 6) return false;
			iteration_offset = upload_x & ~1;
		}
		if (upload_x >= info.width) return false;
		int line_addr = info.vram_addr + ((upload_y * info.vram_width) << (info.vram_size - 1));
		int addr = line_addr + iteration_offset + 4 * (upload_x & 1);
		uint32_t word;
		if ((addr & 3) == 0)
			word = vram32(uint32_t(addr) >> 2);
		else
			word = (uint32_t(vram8(uint32_t(addr) ^ 3)) << 24) | (uint32_t(vram8(uint32_t(addr + 1) ^ 3)) << 16) |
			       (uint32_t(vram8(uint32_t(addr + 2) ^ 3)) << 8) | uint32_t(vram8(uint32_t(addr + 3) ^ 3));
		if (yuv)
		{
			if (upper)
				word = (((word >> 16) & 0xffu) << 8) | (word & 0xffu);
			else
				word = (((word >> 24) & 0xffu) << 8) | ((word >> 8) & 0xffu);
		}
		else
		{
			word >>= 16u - 16u * uint32_t(upper);
			word &= 0xffffu;
		}
		value = word;
		return true;
	}

	bool update_tmem_16(const UploadInfo &info, int tmem16_index, uint32_t &value) const
	{
		int tmem16_offset = (info.tmem_offset & 0xfff) >> 1;
		int stride = info.tmem_stride_words;
		int pixel_offset = (tmem16_index - tmem16_offset) & 0x7ff;
		int upload_x, upload_y, upload_x_xor = 0;
		if (info.mode == MODE_BLOCK)
		{
			int word_offset = pixel_offset >> 2;
			if (info.tmem_stride_words == 0)
				upload_x_xor = (((word_offset * info.dxt) >> 16) & 1) << 1;
			else
			{
				int min_t = compute_upload_t(word_offset, info.min_t_mod);
				int max_t = compute_upload_t(word_offset, info.max_t_mod);
				int max_wc = word_offset - stride * min_t;
				int min_wc = word_offset - stride * max_t;
				min_t = std::max(min_t, (min_wc * info.dxt) >> 16);
				max_t = std::min(max_t, (max_wc * info.dxt) >> 16);
				bool found = false;
				for (int t = max_t; t >= min_t; t--)
				{
					int cand = word_offset - stride * t;
					int ct = (cand * info.dxt) >> 16;
					if (cand + ct * stride == word_offset)
					{
						found = true;
						upload_x_xor = (ct & 1) << 1;
						pixel_offset = (cand << 2) + (pixel_offset & 3);
					}
				}
				if (!found) return false;
			}
			upload_x = pixel_offset;
			upload_y = 0;
		}
		else if (stride == 0)
		{
			upload_x = pixel_offset;
			upload_y = info.height - 1;
		}
		else
		{
			upload_y = compute_upload_t(pixel_offset, info.inv_tmem_stride_words);
			upload_x = pixel_offset - upload_y * stride;
			if (upload_y >= info.height)
			{
				upload_x += stride * (upload_y - info.height + 1);
				upload_y = info.height - 1;
			}
		}
		int iteration_offset = 0;
		if (info.tmem_size != info.vram_size)
		{
			if (info.vram_size - info.tmem_size == 1)
			{
				iteration_offset = (upload_x & ~3) * 4;
				if ((upload_x & ~3) + 2 < (info.vram_effective_width >> (3 - info.vram_size)))
					iteration_offset += 8;
			}
			else if (info.tmem_size == 2 && info.vram_size == 1)
			{
				if (upload_x & 4)
				{
					if ((stride & 4) != 0 && upload_y > 0)
					{
						upload_y--;
						upload_x += stride;
					}
					else
						return false;
				}
				iteration_offset = upload_x & ~3;
			}
		}
		else
			iteration_offset = (upload_x & ~3) * 2;
		if (upload_x >= info.width) return false;
		int line_addr = info.vram_addr + ((upload_y * info.vram_width) << (info.vram_size - 1));
		upload_x ^= ((upload_y & 1) << 1) | upload_x_xor;
		int addr = line_addr + iteration_offset + 2 * (upload_x & 3);
		uint32_t word;
		if ((addr & 1) == 0)
			word = vram16((uint32_t(addr) >> 1) ^ 1u);
		else
			word = (uint32_t(vram8(uint32_t(addr) ^ 3)) << 8) | uint32_t(vram8(uint32_t(addr + 1) ^ 3));
		value = word;
		return true;
	}

	bool update_tmem_lut(const UploadInfo &info, int tmem16_index, uint32_t &value) const
	{
		int tmem16_offset = (info.tmem_offset & 0xfff) >> 1;
		int pixel_offset = (tmem16_index - tmem16_offset) & 0x7ff;
		int splat;
		if (info.vram_size - info.tmem_size == 2)
		{
			splat = pixel_offset >> 2;
			splat <<= info.vram_size - 2;
			if (splat >= info.vram_effective_width) return false;
		}
		else if (info.vram_size - info.tmem_size == 1)
		{
			if ((pixel_offset & 4) == 0)
			{
				int shamt = info.tmem_size + (info.vram_size == 2 ? 2 : 0);
				splat = (pixel_offset & ~7) >> shamt;
				if (splat >= info.vram_effective_width) return false;
			}
			else
				return false;
		}
		else if (info.vram_size == info.tmem_size)
		{
			if ((pixel_offset & 0xc) == 0)
			{
				int shamt = info.tmem_size + (info.vram_size == 2 ? 2 : 0);
				splat = (pixel_offset & ~3) >> shamt;
				if (splat >= info.vram_effective_width) return false;
			}
			else
				return false;
		}
		else if (info.vram_size - info.tmem_size == -1)
		{
			if ((pixel_offset & 0x1c) == 0)
			{
				int shamt = info.tmem_size;
				splat = (pixel_offset >> shamt) & ~7;
				if (splat >= info.vram_effective_width) return false;
			}
			else
				return false;
		}
		else
		{
			int span_iteration = (pixel_offset >> 2) * 2;
			int span_pixel = span_iteration * 2;
			if (span_pixel + 2 < info.vram_effective_width) span_pixel += 2;
			if (span_pixel >= info.vram_effective_width) return false;
			splat = span_pixel;
		}
		int addr = info.vram_addr + (splat << (info.vram_size - 1));
		addr += 2 * (addr & 1) * (pixel_offset & 3);
		uint32_t word;
		if ((addr & 1) == 0)
			word = vram16((uint32_t(addr) >> 1) ^ 1u);
		else
			word = (uint32_t(vram8(uint32_t(addr) ^ 3)) << 8) | uint32_t(vram8(uint32_t(addr + 1) ^ 3));
		value = word;
		return true;
	}

	void apply_upload(const UploadInfo &info)
	{
		uint16_t next[2048];
		for (int gid = 0; gid < 2048; gid++)
		{
			uint32_t value = tmem[gid];
			int idx = gid ^ 1;
			bool upper = idx >= 0x400;
			uint32_t v;
			bool wrote;
			if (info.mode == MODE_TLUT)
				wrote = update_tmem_lut(info, idx, v);
			else
			{
				bool yuv = info.tmem_fmt == FMT_YUV;
				if (info.tmem_size == 3 || yuv) wrote = update_tmem_32(info, idx & 0x3ff, upper, yuv, v);
				else wrote = update_tmem_16(info, idx, v);
			}
			if (wrote) value = v;
			next[gid] = uint16_t(value);
		}
		memcpy(tmem, next, sizeof(tmem));
		tmem_snap.reset();
	}

	// rdp_renderer.cpp:3099-3220 / 3222-3486.
	void load_tile(uint32_t tile, uint32_t slo, uint32_t tlo, uint32_t shi, uint32_t thi, int mode)
	{
		if (upload_needs_flush(texture_image.addr))
		{
			ref.hard();
			end_pass();
		}
		uint32_t tex_addr = texture_image.addr, tex_width = texture_image.width;
		int isize = int(texture_image.size);
		if (mode != MODE_BLOCK)
		{
			if ((thi >> 2) < (tlo >> 2)) return;
			unsigned pc = (((shi >> 2) - (slo >> 2)) + 1) & 0xfff;
			if (!pc) return;
		}
		else
		{
			unsigned pc = ((shi - slo) + 1) & 0xfff;
			if (!pc || pc > 2048) return;
		}
		if (mode == MODE_TILE)
		{
			auto &meta = tiles[tile];
			unsigned ppl = (((shi >> 2) - (slo >> 2)) + 1) & 0xfff;
			unsigned qw = ((ppl << unsigned(meta.size)) + 15) >> 4;
			if (unsigned(meta.size) > unsigned(isize)) qw <<= unsigned(meta.size) - unsigned(isize);
			else if (unsigned(meta.size) < unsigned(isize)) qw >>= unsigned(isize) - unsigned(meta.size);
			unsigned bpl = std::max<unsigned>(qw * 8, meta.stride);
			unsigned max_bpl = 0x1000;
			if (meta.fmt == FMT_YUV) max_bpl /= 2;
			unsigned num_lines = ((thi >> 2) - (tlo >> 2)) + 1;
			unsigned total = bpl * num_lines;
			if (total > max_bpl)
			{
				unsigned mlpi = max_bpl / bpl;
				mlpi &= ~1u;
				if (mlpi == 0) return;
				for (unsigned line = 0; line < num_lines; line += mlpi)
				{
					unsigned n = std::min(num_lines - line, mlpi);
					uint32_t t_lo = tlo + (line << 2);
					uint32_t t_hi = t_lo + ((n - 1) << 2);
					load_tile_iteration(tile, slo, t_lo, shi, t_hi, mode, line * meta.stride, tex_addr, tex_width, isize);
				}
				tiles[tile].slo = slo;
				tiles[tile].shi = shi;
				tiles[tile].tlo = tlo;
				tiles[tile].thi = thi;
				return;
			}
		}
		load_tile_iteration(tile, slo, tlo, shi, thi, mode, 0, tex_addr, tex_width, isize);
	}

	void load_tile_iteration(uint32_t tile, uint32_t slo, uint32_t tlo, uint32_t shi, uint32_t thi, int mode,
	                         uint32_t tmem_offset, uint32_t tex_addr, uint32_t tex_width, int isize)
	{
		auto &meta = tiles[tile];
		meta.slo = slo;
		meta.shi = shi;
		meta.tlo = tlo;
		meta.thi = thi;
		if (meta.fmt == FMT_YUV && (meta.size != 2 || isize != 2)) return;
		if (isize == 0) return;
		if (meta.size == 3 && meta.fmt != FMT_RGBA) return;
		if (mode == MODE_TLUT && meta.size == 3) return;
		if (mode != MODE_TLUT)
		{
			if (isize == 3 && meta.size == 1) return;
			if (isize == 2 && meta.size == 0) return;
			if (isize == 3 && meta.size == 0) return;
		}
		UploadInfo up = {};
		up.tmem_stride_words = int(meta.stride >> 1);
		uint32_t upload_x = 0, upload_y = 0;
		int upload_mode = mode;
		if (upload_mode == MODE_BLOCK)
		{
			upload_x = slo;
			upload_y = tlo;
			unsigned pixel_count = (shi - slo + 1) & 0xfff;
			unsigned dt = thi;
			unsigned max_iter = (pixel_count - 1) >> (4u - unsigned(isize));
			unsigned max_t = (max_iter * dt) >> 11;
			if (max_t != 0)
			{
				unsigned maxn = ((1u << 11u) + dt - 1u) / dt;
				unsigned minn = (1u << 11u) / dt;
				bool uneven = maxn != minn;
				if (uneven)
				{
					unsigned ov = dt * maxn - (1 << 11);
					ov *= max_t;
					if (ov < dt)
					{
						minn = maxn;
						uneven = false;
					}
				}
				up.dxt = int(dt << 5);
				if (meta.size == 3 || meta.fmt == FMT_YUV)
				{
					up.tmem_stride_words <<= 1;
					if (uneven && meta.size != isize) return;
				}
				if (unsigned(meta.size) > unsigned(isize))
				{
					unsigned sh = unsigned(meta.size) - unsigned(isize);
					maxn <<= sh;
					minn <<= sh;
					up.dxt >>= sh;
				}
				else if (unsigned(isize) > unsigned(meta.size))
					return;
				unsigned max_ls = maxn + (unsigned(up.tmem_stride_words) >> 2);
				unsigned min_ls = minn + (unsigned(up.tmem_stride_words) >> 2);
				up.min_t_mod = 1.0f / float(max_ls);
				up.max_t_mod = 1.0f / float(min_ls);
				up.width = int(pixel_count);
				up.height = 1;
				up.tmem_stride_words >>= 2;
			}
			else
			{
				up.width = int(pixel_count);
				up.height = 1;
				up.tmem_stride_words = 0;
				upload_mode = MODE_TILE;
			}
		}
		else
		{
			upload_x = slo >> 2;
			upload_y = tlo >> 2;
			up.width = int((((shi >> 2) - (slo >> 2)) + 1) & 0xfff);
			up.height = int(((thi >> 2) - (tlo >> 2)) + 1);
		}
		if (!up.width) return;
		switch (isize)
		{
		case 1: up.vram_effective_width = (up.width + 7) & ~7; break;
		case 2: up.vram_effective_width = upload_mode == MODE_TLUT ? up.width : ((up.width + 3) & ~3); break;
		case 3: up.vram_effective_width = (up.width + 1) & ~1; break;
		default: break;
		}
		switch (meta.size)
		{
		case 0: up.width = ((up.width + 15) & ~15) >> 2; break;
		case 1: up.width = ((up.width + 7) & ~7) >> 1; break;
		case 2:
			up.width = (up.width + 3) & ~3;
			if (meta.fmt == FMT_YUV) up.width >>= 1;
			break;
		default: up.width = (up.width + 1) & ~1; break;
		}
		if (up.height > 1 && upload_mode == MODE_TLUT) return;
		up.vram_addr = int(tex_addr + ((tex_width * upload_y + upload_x) << (unsigned(isize) - 1)));
		up.vram_width = upload_mode == MODE_BLOCK ? up.vram_effective_width : int(tex_width);
		up.vram_size = isize;
		up.tmem_offset = int((meta.offset + tmem_offset) & 0xfff);
		up.tmem_size = meta.size;
		up.tmem_fmt = meta.fmt;
		up.mode = upload_mode;
		up.inv_tmem_stride_words = 1.0f / float(up.tmem_stride_words);
		apply_upload(up);
		ref.upload();
		if (++pass_uploads + 1 >= 256) end_pass();
	}

	// ======================================================================= commands
	static uint32_t cmd_length(uint32_t op)
	{
		switch (op)
		{
		case 0x08: return 8;
		case 0x09: return 12;
		case 0x0a: return 24;
		case 0x0b: return 28;
		case 0x0c: return 24;
		case 0x0d: return 28;
		case 0x0e: return 40;
		case 0x0f: return 44;
		case 0x24: case 0x25: return 4;
		default: return 2;
		}
	}

	void set_other_modes(const uint32_t *w)
	{
		auto m = [](uint32_t &f, bool on, uint32_t bit) { if (on) f |= bit; else f &= ~bit; };
		uint32_t &sf = static_state.flags;
		uint32_t &df = depth_blend.flags;
		m(sf, w[0] & (1 << 19), R_PERSPECTIVE);
		m(sf, w[0] & (1 << 18), R_DETAIL);
		m(sf, w[0] & (1 << 17), R_SHARPEN);
		m(sf, w[0] & (1 << 16), R_TEX_LOD);
		m(sf, w[0] & (1 << 15), R_TLUT);
		m(sf, w[0] & (1 << 14), R_TLUT_TYPE);
		m(sf, w[0] & (1 << 13), R_SAMPLE_QUAD);
		m(sf, w[0] & (1 << 12), R_MID_TEXEL);
		m(sf, w[0] & (1 << 11), R_BILERP0);
		m(sf, w[0] & (1 << 10), R_BILERP1);
		m(sf, w[0] & (1 << 9), R_CONVERT_ONE);
		m(df, w[1] & (1 << 14), DB_FORCE_BLEND);
		m(sf, w[1] & (1 << 13), R_ALPHA_CVG_SELECT);
		m(sf, w[1] & (1 << 12), R_CVG_TIMES_ALPHA);
		m(df, w[1] & (1 << 7), DB_COLOR_ON_CVG);
		m(df, w[1] & (1 << 6), DB_IMAGE_READ);
		m(df, w[1] & (1 << 5), DB_DEPTH_UPDATE);
		m(df, w[1] & (1 << 4), DB_DEPTH_TEST);
		m(sf, w[1] & (1 << 3), R_AA);
		m(df, w[1] & (1 << 3), DB_AA);
		m(sf, w[1] & (1 << 1), R_ALPHA_TEST_DITHER);
		m(sf, w[1] & (1 << 0), R_ALPHA_TEST);
		static_state.dither = int((w[0] >> 4) & 0x0f);
		m(df, (static_state.dither >> 2) != 3, DB_DITHER);
		depth_blend.coverage_mode = int((w[1] >> 8) & 3);
		depth_blend.z_mode = int((w[1] >> 10) & 3);
		sf &= ~(R_MULTI_CYCLE | R_FILL | R_COPY);
		df &= ~DB_MULTI_CYCLE;
		switch ((w[0] >> 20) & 3)
		{
		case 1: sf |= R_MULTI_CYCLE; df |= DB_MULTI_CYCLE; break;
		case 3: sf |= R_FILL; break;
		case 2: sf |= R_COPY; break;
		default: break;
		}
		depth_blend.cyc[0].m1a = int((w[1] >> 30) & 3);
		depth_blend.cyc[1].m1a = int((w[1] >> 28) & 3);
		depth_blend.cyc[0].m1b = int((w[1] >> 26) & 3);
		depth_blend.cyc[1].m1b = int((w[1] >> 24) & 3);
		depth_blend.cyc[0].m2a = int((w[1] >> 22) & 3);
		depth_blend.cyc[1].m2a = int((w[1] >> 20) & 3);
		depth_blend.cyc[0].m2b = int((w[1] >> 18) & 3);
		depth_blend.cyc[1].m2b = int((w[1] >> 16) & 3);
		constants.use_prim_depth = (w[1] & (1 << 2)) != 0;
	}

	void set_combine(const uint32_t *w)
	{
		auto &st = static_state;
		st.rgb[0][0] = int((w[0] >> 20) & 0xf);
		st.rgb[0][2] = int((w[0] >> 15) & 0x1f);
		st.rgb[0][1] = int((w[1] >> 28) & 0xf);
		st.rgb[0][3] = int((w[1] >> 15) & 0x7);
		st.alpha[0][0] = int((w[0] >> 12) & 0x7);
		st.alpha[0][1] = int((w[1] >> 12) & 0x7);
		st.alpha[0][2] = int((w[0] >> 9) & 0x7);
		st.alpha[0][3] = int((w[1] >> 9) & 0x7);
		st.rgb[1][0] = int((w[0] >> 5) & 0xf);
		st.rgb[1][2] = int((w[0] >> 0) & 0x1f);
		st.rgb[1][1] = int((w[1] >> 24) & 0xf);
		st.rgb[1][3] = int((w[1] >> 6) & 0x7);
		st.alpha[1][0] = int((w[1] >> 21) & 0x7);
		st.alpha[1][1] = int((w[1] >> 3) & 0x7);
		st.alpha[1][2] = int((w[1] >> 18) & 0x7);
		st.alpha[1][3] = int((w[1] >> 0) & 0x7);
	}

	void set_tile(const uint32_t *w)
	{
		uint32_t t = (w[1] >> 24) & 7;
		TileInfo &ti = tiles[t];
		ti.offset = ((w[0] >> 0) & 511) << 3;
		ti.stride = ((w[0] >> 9) & 511) << 3;
		ti.size = int((w[0] >> 19) & 3);
		ti.fmt = int((w[0] >> 21) & 7);
		ti.palette = int((w[1] >> 20) & 15);
		ti.shift_s = int((w[1] >> 0) & 15);
		ti.mask_s = int((w[1] >> 4) & 15);
		ti.shift_t = int((w[1] >> 10) & 15);
		ti.mask_t = int((w[1] >> 14) & 15);
		ti.flags = 0;
		if (w[1] & (1 << 8)) ti.flags |= TILE_MIRROR_S;
		if (w[1] & (1 << 9)) ti.flags |= TILE_CLAMP_S;
		if (w[1] & (1 << 18)) ti.flags |= TILE_MIRROR_T;
		if (w[1] & (1 << 19)) ti.flags |= TILE_CLAMP_T;
		if (ti.mask_s > 10) ti.mask_s = 10;
		else if (ti.mask_s == 0) ti.flags |= TILE_CLAMP_S;
		if (ti.mask_t > 10) ti.mask_t = 10;
		else if (ti.mask_t == 0) ti.flags |= TILE_CLAMP_T;
	}

	void rect(const uint32_t *w, bool textured, bool flip_rect)
	{
		uint32_t xl = (w[0] >> 12) & 0xfff, yl = w[0] & 0xfff, xh = (w[1] >> 12) & 0xfff, yh = w[1] & 0xfff;
		if (static_state.flags & (R_COPY | R_FILL)) yl |= 3;
		TriSetup s = {};
		Attr a = {};
		s.xh = int(xh << 13);
		s.xl = int(xl << 13);
		s.xm = int(xl << 13);
		s.ym = int(yl);
		s.yl = int(yl);
		s.yh = int(yh);
		s.flags = TRI_FLIP | TRI_DISABLE_UPSCALING;
		if (textured)
		{
			uint32_t tile = (w[1] >> 24) & 7;
			int sv = int((w[2] >> 16) & 0xffff), tv = int(w[2] & 0xffff);
			int dsdx = bfe_s(int((w[3] >> 16) & 0xffff), 16), dtdy = bfe_s(int(w[3] & 0xffff), 16);
			s.flags = TRI_FLIP | (flip_rect ? TRI_DISABLE_UPSCALING : 0) | ((quirks & 0xffu) ? TRI_DISABLE_UPSCALING : 0) |
			          ((quirks & 0xff00u) ? TRI_NATIVE_LOD : 0);
			s.tile = tile;
			a.stzw[0] = sv << 16;
			a.stzw[1] = tv << 16;
			if (!flip_rect)
			{
				a.dstzw_dx[0] = dsdx << 11;
				a.dstzw_de[1] = dtdy << 11;
				a.dstzw_dy[1] = dtdy << 11;
			}
			else
			{
				a.dstzw_dx[1] = dtdy << 11;
				a.dstzw_de[0] = dsdx << 11;
				a.dstzw_dy[0] = dsdx << 11;
			}
			if (static_state.flags & R_COPY) s.flags |= TRI_SKIP_XFRAC;
		}
		draw_primitive(s, a);
	}

	void command(const uint32_t *w)
	{
		uint32_t op = (w[0] >> 24) & 63;
		switch (op)
		{
		case 0x04: quirks = w[1]; break;
		case 0x08: case 0x09: case 0x0a: case 0x0b: case 0x0c: case 0x0d: case 0x0e: case 0x0f:
		{
			TriSetup s;
			Attr a = {};
			decode_triangle_setup(s, w);
			const uint32_t *p = w + 8;
			bool shade = (op & 4) != 0, tex = (op & 2) != 0, z = (op & 1) != 0;
			if (shade) { decode_rgba(a, p); p += 16; }
			if (tex) { decode_tex(a, p); p += 16; }
			if (z) decode_z(a, p);
			draw_primitive(s, a);
			break;
		}
		case 0x24: rect(w, true, false); break;
		case 0x25: rect(w, true, true); break;
		case 0x2a:
			constants.key_width[1] = int((w[0] >> 12) & 0xfff);
			constants.key_width[2] = int(w[0] & 0xfff);
			constants.key_center[1] = int((w[1] >> 24) & 0xff);
			constants.key_scale[1] = int((w[1] >> 16) & 0xff);
			constants.key_center[2] = int((w[1] >> 8) & 0xff);
			constants.key_scale[2] = int(w[1] & 0xff);
			break;
		case 0x2b:
			constants.key_width[0] = int((w[1] >> 16) & 0xfff);
			constants.key_center[0] = int((w[1] >> 8) & 0xff);
			constants.key_scale[0] = int(w[1] & 0xff);
			break;
		case 0x2c:
		{
			uint64_t m = (uint64_t(w[0]) << 32) | w[1];
			int k[6];
			for (int i = 0; i < 6; i++) k[i] = int((m >> (45 - 9 * i)) & 0x1ff);
			for (int i = 0; i < 4; i++) constants.convert[i] = 2 * bfe_s(k[i], 9) + 1;
			constants.convert[4] = k[4];
			constants.convert[5] = k[5];
			break;
		}
		case 0x2d:
			scissor.xlo = int((w[0] >> 12) & 0xfff);
			scissor.xhi = int((w[1] >> 12) & 0xfff);
			scissor.ylo = int(w[0] & 0xfff);
			scissor.yhi = int(w[1] & 0xfff);
			if (w[1] & (1 << 25)) static_state.flags |= R_INTERLACE_FIELD; else static_state.flags &= ~R_INTERLACE_FIELD;
			if (w[1] & (1 << 24)) static_state.flags |= R_INTERLACE_KEEP_ODD; else static_state.flags &= ~R_INTERLACE_KEEP_ODD;
			break;
		case 0x2e:
			constants.prim_depth = int((w[1] >> 16) & 0x7fff) << 16;
			constants.prim_dz = int(w[1] & 0xffff);
			break;
		case 0x2f:
			raw_other_modes[0] = w[0];
			raw_other_modes[1] = w[1];
			set_other_modes(w);
			break;
		case 0x30: load_tile((w[1] >> 24) & 7, (w[0] >> 12) & 0xfff, w[0] & 0xfff, (w[1] >> 12) & 0xfff, w[1] & 0xfff, MODE_TLUT); break;
		case 0x32:
		{
			uint32_t t = (w[1] >> 24) & 7;
			tiles[t].slo = (w[0] >> 12) & 0xfff;
			tiles[t].shi = (w[1] >> 12) & 0xfff;
			tiles[t].tlo = w[0] & 0xfff;
			tiles[t].thi = w[1] & 0xfff;
			break;
		}
		case 0x33: load_tile((w[1] >> 24) & 7, (w[0] >> 12) & 0xfff, w[0] & 0xfff, (w[1] >> 12) & 0xfff, w[1] & 0xfff, MODE_BLOCK); break;
		case 0x34: load_tile((w[1] >> 24) & 7, (w[0] >> 12) & 0xfff, w[0] & 0xfff, (w[1] >> 12) & 0xfff, w[1] & 0xfff, MODE_TILE); break;
		case 0x35: set_tile(w); break;
		case 0x36: rect(w, false, false); break;
		case 0x37: constants.fill_color = w[1]; break;
		case 0x38: constants.fog_color = w[1]; break;
		case 0x39: constants.blend_color = w[1]; break;
		case 0x3a:
			constants.min_level = int((w[0] >> 8) & 31);
			constants.prim_lod_frac = int(w[0] & 0xff);
			constants.primitive_color = w[1];
			break;
		case 0x3b: constants.env_color = w[1]; break;
		case 0x3c:
			raw_combine[0] = w[0];
			raw_combine[1] = w[1];
			set_combine(w);
			break;
		case 0x3d:
			texture_image.fmt = int((w[0] >> 21) & 7);
			texture_image.size = (w[0] >> 19) & 3;
			texture_image.width = (w[0] & 0x3ff) + 1;
			texture_image.addr = w[1] & 0xffffff;
			break;
		case 0x29:
			ref.hard();
			end_pass();
			break;
		case 0x3e:
			if ((w[1] & 0xffffff) != fb.depth_addr)
			{
				ref.hard();
				end_pass();
			}
			fb.depth_addr = w[1] & 0xffffff;
			break;
		case 0x3f:
		{
			uint32_t f = (w[0] >> 21) & 7, sz = (w[0] >> 19) & 3;
			uint32_t width = (w[0] & 1023) + 1, addr = w[1] & 0xffffff;
			int fmt;
			switch (sz)
			{
			case 0: fmt = FB_I4; break;
			case 1: fmt = FB_I8; break;
			case 2: fmt = f ? FB_IA88 : FB_RGBA5551; break;
			default: fmt = FB_RGBA8888; break;
			}
			if (width != fb.width || addr != fb.addr || fmt != fb.fmt)
			{
				ref.hard();
				end_pass();
			}
			fb.width = width;
			fb.addr = addr;
			fb.fmt = fmt;
			break;
		}
		default:
			break;
		}
	}
};

} // namespace

// ============================================================================ C API
extern "C" {

void *oracle_create(uint32_t rdram_size, uint32_t hidden_size)
{
	if (rdram_size == 0 || (rdram_size & (rdram_size - 1)) || hidden_size == 0 || (hidden_size & (hidden_size - 1)))
		return nullptr;
	Oracle *o = new Oracle();
	o->rdram_size = rdram_size;
	o->hidden_size = hidden_size;
	o->rdram.assign(rdram_size, 0);
	o->pixel_cache.assign(1024 * 1024, PixelStateSlot{});
	o->hidden.assign(hidden_size, 0x03);
	o->mem_rd = o->rdram.data();
	o->mem_hd = o->hidden.data();
	o->init_luts();
	return o;
}

void oracle_vi_destroy(void *vi);
void oracle_destroy(void *h)
{
	Oracle *o = static_cast<Oracle *>(h);
	if (o->vi_state) oracle_vi_destroy(o->vi_state);
	delete o;
}
uint32_t oracle_rdram_size(void *h) { return static_cast<Oracle *>(h)->rdram_size; }
uint32_t oracle_hidden_size(void *h) { return static_cast<Oracle *>(h)->hidden_size; }
void *oracle_vi_state(void *h) { return static_cast<Oracle *>(h)->vi_state; }
void oracle_set_vi_state(void *h, void *vi) { static_cast<Oracle *>(h)->vi_state = vi; }

void oracle_write_rdram(void *h, const uint8_t *data, uint32_t offset, uint32_t size)
{
	Oracle *o = static_cast<Oracle *>(h);
	memcpy(o->rdram.data() + offset, data, size);
}
void oracle_read_rdram(void *h, uint8_t *data, uint32_t offset, uint32_t size)
{
	Oracle *o = static_cast<Oracle *>(h);
	o->end_pass();
	memcpy(data, o->rdram.data() + offset, size);
}
void oracle_read_hidden(void *h, uint8_t *data, uint32_t offset, uint32_t size)
{
	Oracle *o = static_cast<Oracle *>(h);
	o->end_pass();
	memcpy(data, o->hidden.data() + offset, size);
}
// Internal upscaling (factor 1, 2, 4 or 8) with optional super-sampled readback and its dither;
// set before the first command.  Returns 0, or -1 for an unsupported factor or a hidden RDRAM
// that is not half of RDRAM.
int oracle_set_upscaling(void *h, uint32_t factor, uint32_t super_sampled, uint32_t dither)
{
	Oracle *o = static_cast<Oracle *>(h);
	return o->set_upscaling(int(factor), super_sampled != 0, dither != 0) ? 0 : -1;
}
uint32_t oracle_upscaling_factor(void *h) { return 1u << static_cast<Oracle *>(h)->up_log2; }
// The multisampled copies (factor^2 slices of RDRAM / hidden RDRAM); byte offsets.
void oracle_read_upscaled_rdram(void *h, uint8_t *data, uint64_t offset, uint64_t size)
{
	Oracle *o = static_cast<Oracle *>(h);
	o->end_pass();
	memcpy(data, o->ms_rdram.data() + offset, size_t(size));
}
void oracle_read_upscaled_hidden(void *h, uint8_t *data, uint64_t offset, uint64_t size)
{
	Oracle *o = static_cast<Oracle *>(h);
	o->end_pass();
	memcpy(data, o->ms_hidden.data() + offset, size_t(size));
}
// The "pre" update of the upscaled domain over a scanout range (VideoInterface::vram_fetch_stage,
// video_interface.cpp:412-420): `length` elements of 2^psl2 bytes from `offset`.
void oracle_upscale_pre_external(void *h, uint32_t offset, uint32_t length, uint32_t psl2)
{
	Oracle *o = static_cast<Oracle *>(h);
	o->end_pass();
	if (o->up_log2) o->upscale_range(offset, offset, length, int(psl2), false);
}

void oracle_write_hidden(void *h, const uint8_t *data, uint32_t offset, uint32_t size)
{
	Oracle *o = static_cast<Oracle *>(h);
	memcpy(o->hidden.data() + offset, data, size);
}
void oracle_read_tmem(void *h, uint16_t *out)
{
	Oracle *o = static_cast<Oracle *>(h);
	memcpy(out, o->tmem, sizeof(o->tmem));
}

// Processes a stream of RDP command words.  Returns the number of words consumed
// (a trailing partial command is left unconsumed).
uint32_t oracle_enqueue(void *h, const uint32_t *words, uint32_t num_words)
{
	Oracle *o = static_cast<Oracle *>(h);
	uint32_t i = 0;
	while (i < num_words)
	{
		uint32_t op = (words[i] >> 24) & 63;
		uint32_t len = Oracle::cmd_length(op);
		if (i + len > num_words) break;
		o->command(words + i);
		i += len;
	}
	return i;
}

// Applies caller-made upload plans (64-byte records: the UploadInfo fields, then 4 bytes of
// padding) to the oracle's TMEM in order, as tmem_update.comp applies a pass's uploads.  Tests use
// it to check hand-derived plans against the plans the oracle derives from load commands.
void oracle_apply_upload_plans(void *h, const uint8_t *plans, uint32_t count)
{
	static_assert(sizeof(UploadInfo) == 60, "UploadInfo is the plan record without its padding");
	Oracle *o = static_cast<Oracle *>(h);
	for (uint32_t i = 0; i < count; i++)
	{
		UploadInfo u;
		memcpy(&u, plans + size_t(i) * 64, sizeof(u));
		o->apply_upload(u);
	}
}

uint64_t oracle_fragments(void *h) { return static_cast<Oracle *>(h)->fragments; }
uint32_t oracle_primitive_count(void *h) { return static_cast<Oracle *>(h)->primitive_counter; }
uint64_t oracle_reference_passes(void *h) { return static_cast<Oracle *>(h)->ref.total(); }

void oracle_blender_lut(void *h, uint8_t *out)
{
	memcpy(out, static_cast<Oracle *>(h)->blender_lut, 0x8000);
}

// Known-answer hooks for the fixed-point primitives.
int oracle_z_compress(int z) { return Oracle::z_compress(z); }
int oracle_z_decompress(int z) { return Oracle::z_decompress(z); }
int oracle_dz_compress(int dz) { return Oracle::dz_compress_host(dz); }
int oracle_clamp_9bit(int v) { return Oracle::clamp_9bit_notrunc(v); }
int oracle_clamp_z(int v) { return Oracle::clamp_z(v); }
void oracle_perspective_divide(int s, int t, int w, int *out_st, int *overflow)
{
	int stw[3] = { s, t, w };
	bool ov = false;
	Oracle::perspective_divide(stw, out_st, ov);
	*overflow = ov ? 1 : 0;
}
int oracle_noise(uint32_t x, uint32_t y, uint32_t p)
{
	Oracle o;
	o.reseed_noise(x, y, p);
	return int(o.seeded_noise);
}
}
