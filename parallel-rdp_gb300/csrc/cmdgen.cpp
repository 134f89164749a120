/*
 * Seeded synthetic RDP command-stream generator (input synthesis for tests and
 * benchmarks; not part of the rendering path).
 *
 * It plays the role of the reference's CommandBuilder / triangle converter
 * (rdp_command_builder.cpp:278-750, triangle_converter.cpp:129-273): it turns
 * randomly drawn primitives into raw 32-bit RDP command words.  The word
 * layouts are the RDP's own (decoded by rdp_device.cpp:268-864); the triangle
 * set-up arithmetic (edge slopes, attribute planes) is this project's own.
 *
 * Everything is driven by a private xoshiro256** generator so that a seed
 * always produces the same words on every host.
 */
#include <stdint.h>
#include <string.h>
#include <math.h>
#include <vector>
#include <algorithm>

#include "../../include/rdp_cmdgen.h"

namespace {

// Every draw from the generator's RNG is its own statement: the order in which C++
// evaluates function arguments and operands is unspecified and differs between
// compilers and targets, and the streams must be identical on every host.
struct Rng
{
	uint64_t s[4];
	explicit Rng(uint64_t seed)
	{
		uint64_t z = seed + 0x9e3779b97f4a7c15ull;
		for (int i = 0; i < 4; i++)
		{
			z += 0x9e3779b97f4a7c15ull;
			uint64_t x = z;
			x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
			x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
			s[i] = x ^ (x >> 31);
		}
	}
	static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
	uint64_t next()
	{
		uint64_t r = rotl(s[1] * 5, 7) * 9;
		uint64_t t = s[1] << 17;
		s[2] ^= s[0];
		s[3] ^= s[1];
		s[1] ^= s[2];
		s[0] ^= s[3];
		s[2] ^= t;
		s[3] = rotl(s[3], 45);
		return r;
	}
	uint32_t u32() { return uint32_t(next() >> 32); }
	uint32_t below(uint32_t n) { return n ? uint32_t((uint64_t(u32()) * n) >> 32) : 0; }
	double uniform() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
	double normal()
	{
		double u1 = std::max(uniform(), 1e-300), u2 = uniform();
		return sqrt(-2.0 * det_log(u1)) * det_cos(6.283185307179586 * u2);
	}

	// exp / log / cos from their series with only +, -, *, / and exact scaling, so
	// that the generated streams are identical on every host (libm results and FMA
	// contraction differ between x86-64 and AArch64).
	static double det_exp(double x)
	{
		const double ln2 = 0.6931471805599453;
		double k = floor(x / ln2 + 0.5);
		double r = x - k * ln2, term = 1.0, sum = 1.0;
		for (int n = 1; n < 24; n++)
		{
			term = term * r / double(n);
			sum += term;
		}
		return ldexp(sum, int(k));
	}
	static double det_log(double x)
	{
		int e;
		double m = frexp(x, &e); // x = m * 2^e, m in [0.5, 1)
		if (m < 0.7071067811865476)
		{
			m *= 2.0;
			e -= 1;
		}
		double z = (m - 1.0) / (m + 1.0), z2 = z * z, term = z, sum = 0.0;
		for (int n = 1; n < 60; n += 2)
		{
			sum += term / double(n);
			term *= z2;
		}
		return 2.0 * sum + double(e) * 0.6931471805599453;
	}
	static double det_cos(double a)
	{
		const double two_pi = 6.283185307179586;
		a -= two_pi * floor(a / two_pi + 0.5); // [-pi, pi]
		double a2 = a * a, term = 1.0, sum = 1.0;
		for (int n = 2; n < 40; n += 2)
		{
			term = -term * a2 / (double(n - 1) * double(n));
			sum += term;
		}
		return sum;
	}
};

static inline int32_t to_fixed16(double v)
{
	double r = floor(v * 65536.0 + 0.5);
	if (r > 2147483647.0) r = 2147483647.0;
	if (r < -2147483648.0) r = -2147483648.0;
	return int32_t(int64_t(r));
}

// RDP op codes.
enum
{
	OP_TRI = 0x08, OP_TEXRECT = 0x24, OP_SYNC_LOAD = 0x26, OP_SYNC_PIPE = 0x27, OP_SYNC_TILE = 0x28,
	OP_SYNC_FULL = 0x29, OP_SET_CONVERT = 0x2c, OP_SET_SCISSOR = 0x2d, OP_SET_PRIM_DEPTH = 0x2e,
	OP_SET_OTHER_MODES = 0x2f, OP_LOAD_TLUT = 0x30, OP_SET_TILE_SIZE = 0x32, OP_LOAD_BLOCK = 0x33,
	OP_LOAD_TILE = 0x34, OP_SET_TILE = 0x35, OP_FILL_RECT = 0x36, OP_SET_FILL_COLOR = 0x37,
	OP_SET_FOG_COLOR = 0x38, OP_SET_BLEND_COLOR = 0x39, OP_SET_PRIM_COLOR = 0x3a, OP_SET_ENV_COLOR = 0x3b,
	OP_SET_COMBINE = 0x3c, OP_SET_TEXTURE_IMAGE = 0x3d, OP_SET_MASK_IMAGE = 0x3e, OP_SET_COLOR_IMAGE = 0x3f
};

// Other-modes bit helpers (word 0 = high, word 1 = low), decoded by rdp_device.cpp:474-540.
struct OtherModes
{
	uint32_t cycle = 0;       // 0: 1-cycle, 1: 2-cycle, 2: copy, 3: fill
	bool persp = false, detail = false, sharpen = false, tex_lod = false, tlut = false, tlut_ia = false;
	bool sample_quad = false, mid_texel = false, bilerp0 = true, bilerp1 = true, convert_one = false;
	uint32_t rgb_dither = 3, alpha_dither = 3;
	uint32_t blend[2][4] = { { 0, 0, 0, 0 }, { 0, 0, 0, 0 } }; // m1a, m1b, m2a, m2b per cycle
	bool force_blend = false, alpha_cvg_select = false, cvg_times_alpha = false;
	uint32_t z_mode = 0, cvg_mode = 0;
	bool color_on_cvg = false, image_read = false, z_update = false, z_compare = false, aa = false;
	bool prim_depth = false, alpha_test_dither = false, alpha_test = false;

	void encode(uint32_t w[2]) const
	{
		uint32_t h = uint32_t(OP_SET_OTHER_MODES) << 24;
		h |= (cycle & 3) << 20;
		h |= persp ? 1u << 19 : 0;
		h |= detail ? 1u << 18 : 0;
		h |= sharpen ? 1u << 17 : 0;
		h |= tex_lod ? 1u << 16 : 0;
		h |= tlut ? 1u << 15 : 0;
		h |= tlut_ia ? 1u << 14 : 0;
		h |= sample_quad ? 1u << 13 : 0;
		h |= mid_texel ? 1u << 12 : 0;
		h |= bilerp0 ? 1u << 11 : 0;
		h |= bilerp1 ? 1u << 10 : 0;
		h |= convert_one ? 1u << 9 : 0;
		h |= (rgb_dither & 3) << 6;
		h |= (alpha_dither & 3) << 4;
		uint32_t l = 0;
		l |= (blend[0][0] & 3) << 30;
		l |= (blend[1][0] & 3) << 28;
		l |= (blend[0][1] & 3) << 26;
		l |= (blend[1][1] & 3) << 24;
		l |= (blend[0][2] & 3) << 22;
		l |= (blend[1][2] & 3) << 20;
		l |= (blend[0][3] & 3) << 18;
		l |= (blend[1][3] & 3) << 16;
		l |= force_blend ? 1u << 14 : 0;
		l |= alpha_cvg_select ? 1u << 13 : 0;
		l |= cvg_times_alpha ? 1u << 12 : 0;
		l |= (z_mode & 3) << 10;
		l |= (cvg_mode & 3) << 8;
		l |= color_on_cvg ? 1u << 7 : 0;
		l |= image_read ? 1u << 6 : 0;
		l |= z_update ? 1u << 5 : 0;
		l |= z_compare ? 1u << 4 : 0;
		l |= aa ? 1u << 3 : 0;
		l |= prim_depth ? 1u << 2 : 0;
		l |= alpha_test_dither ? 1u << 1 : 0;
		l |= alpha_test ? 1u << 0 : 0;
		w[0] = h;
		w[1] = l;
	}
};

struct Combiner
{
	// [cycle][muladd, mulsub, mul, add]
	uint32_t rgb[2][4];
	uint32_t alpha[2][4];
	void encode(uint32_t w[2]) const
	{
		uint32_t h = uint32_t(OP_SET_COMBINE) << 24;
		h |= (rgb[0][0] & 0xf) << 20;
		h |= (rgb[0][2] & 0x1f) << 15;
		h |= (alpha[0][0] & 7) << 12;
		h |= (alpha[0][2] & 7) << 9;
		h |= (rgb[1][0] & 0xf) << 5;
		h |= (rgb[1][2] & 0x1f) << 0;
		uint32_t l = 0;
		l |= (rgb[0][1] & 0xf) << 28;
		l |= (rgb[1][1] & 0xf) << 24;
		l |= (alpha[1][0] & 7) << 21;
		l |= (alpha[1][2] & 7) << 18;
		l |= (rgb[0][3] & 7) << 15;
		l |= (alpha[0][1] & 7) << 12;
		l |= (alpha[0][3] & 7) << 9;
		l |= (rgb[1][3] & 7) << 6;
		l |= (alpha[1][1] & 7) << 3;
		l |= (alpha[1][3] & 7) << 0;
		w[0] = h;
		w[1] = l;
	}
};

struct Vertex
{
	double x, y;      // pixels
	double c[4];      // 0..255
	double z;         // 0..32767
	double s, t, w;   // texel*32 (already multiplied by w), w in (0,1]
};

struct Gen
{
	rdpgen_params p;
	Rng rng;
	std::vector<uint32_t> words;
	std::vector<uint32_t> frame_begin; // word index where each frame's prologue starts
	struct Blob { uint32_t addr; std::vector<uint8_t> bytes; };
	std::vector<Blob> blobs;
	uint32_t prims = 0;
	uint32_t frame_prims_begin = 0;

	// RDRAM layout.
	static constexpr uint32_t COLOR_ADDR = 0x100000;
	static constexpr uint32_t DEPTH_ADDR = 0x300000;
	static constexpr uint32_t LAYER_ADDR = 0x480000;
	static constexpr uint32_t TEX_ADDR = 0x600000;
	static constexpr uint32_t NUM_TEX = 8;
	// Texture blob layout (per texture slot k): RGBA16 32x32 (2 KiB) + mip 16x16 (512 B) + 8x8 (128 B)
	// at TEX_ADDR + k*0x1000; CI8 32x32 (1 KiB) at TEX_ADDR + 0x10000 + k*0x400;
	// TLUT (256 x RGBA16 = 512 B) at TEX_ADDR + 0x20000 + k*0x200.

	explicit Gen(const rdpgen_params &params) : p(params), rng(uint64_t(params.seed) * 0x100000001b3ull + 17) {}

	void emit(const uint32_t *w, int n) { words.insert(words.end(), w, w + n); }
	void emit2(uint32_t a, uint32_t b) { words.push_back(a); words.push_back(b); }

	uint32_t fb_size_bits() const
	{
		switch (p.fb_format)
		{
		case RDPGEN_FB_RGBA8888: return 3;
		case RDPGEN_FB_I8: return 1;
		case RDPGEN_FB_I4: return 0;
		default: return 2;
		}
	}
	uint32_t fb_fmt_bits() const { return p.fb_format == RDPGEN_FB_IA88 ? 3u : 0u; }

	void set_color_image(uint32_t addr, uint32_t size_bits, uint32_t width, uint32_t fmt_bits = 0)
	{
		emit2((uint32_t(OP_SET_COLOR_IMAGE) << 24) | (fmt_bits << 21) | (size_bits << 19) | ((width - 1) & 1023),
		      addr & 0xffffff);
	}
	void set_scissor(uint32_t w, uint32_t h)
	{
		emit2((uint32_t(OP_SET_SCISSOR) << 24) | (0 << 12) | 0, ((w << 2) << 12) | (h << 2));
	}
	void set_other_modes(const OtherModes &om)
	{
		uint32_t w[2];
		om.encode(w);
		emit(w, 2);
	}
	void set_combiner(const Combiner &c)
	{
		uint32_t w[2];
		c.encode(w);
		emit(w, 2);
	}
	void fill_rect(uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1)
	{
		// Coordinates in 10.2; x1/y1 exclusive-ish (fill mode forces yl |= 3).
		emit2((uint32_t(OP_FILL_RECT) << 24) | ((x1 & 0xfff) << 12) | (y1 & 0xfff), ((x0 & 0xfff) << 12) | (y0 & 0xfff));
	}
	void color_reg(uint32_t op, uint32_t rgba) { emit2(uint32_t(op) << 24, rgba); }
	void set_texture_image(uint32_t addr, uint32_t fmt, uint32_t size_bits, uint32_t width)
	{
		emit2((uint32_t(OP_SET_TEXTURE_IMAGE) << 24) | (fmt << 21) | (size_bits << 19) | ((width - 1) & 0x3ff), addr & 0xffffff);
	}
	void set_tile(uint32_t tile, uint32_t fmt, uint32_t size_bits, uint32_t line_qw, uint32_t tmem_qw, uint32_t palette,
	              uint32_t cm_t, uint32_t mask_t, uint32_t shift_t, uint32_t cm_s, uint32_t mask_s, uint32_t shift_s)
	{
		uint32_t h = (uint32_t(OP_SET_TILE) << 24) | (fmt << 21) | (size_bits << 19) | ((line_qw & 511) << 9) | (tmem_qw & 511);
		uint32_t l = ((tile & 7) << 24) | ((palette & 15) << 20) | ((cm_t & 3) << 18) | ((mask_t & 15) << 14) |
		             ((shift_t & 15) << 10) | ((cm_s & 3) << 8) | ((mask_s & 15) << 4) | (shift_s & 15);
		emit2(h, l);
	}
	void tile_cmd(uint32_t op, uint32_t tile, uint32_t sl, uint32_t tl, uint32_t sh, uint32_t th)
	{
		emit2((uint32_t(op) << 24) | ((sl & 0xfff) << 12) | (tl & 0xfff), ((tile & 7) << 24) | ((sh & 0xfff) << 12) | (th & 0xfff));
	}

	// ------------------------------------------------------------------ textures in RDRAM
	void make_textures()
	{
		for (uint32_t k = 0; k < NUM_TEX; k++)
		{
			Blob b;
			b.addr = TEX_ADDR + k * 0x1000;
			b.bytes.resize(2048 + 512 + 128);
			for (auto &v : b.bytes) v = uint8_t(rng.u32());
			blobs.push_back(std::move(b));
			Blob ci;
			ci.addr = TEX_ADDR + 0x10000 + k * 0x400;
			ci.bytes.resize(1024);
			for (auto &v : ci.bytes) v = uint8_t(rng.u32());
			blobs.push_back(std::move(ci));
			Blob lut;
			lut.addr = TEX_ADDR + 0x20000 + k * 0x200;
			lut.bytes.resize(512);
			for (auto &v : lut.bytes) v = uint8_t(rng.u32());
			blobs.push_back(std::move(lut));
		}
	}

	// ------------------------------------------------------------------ triangle emission
	bool emit_triangle(Vertex v[3], bool shade, bool tex, bool z, uint32_t tile, uint32_t max_level)
	{
		// Quantise to 10.2 fixed point.
		int xs[3], ys[3];
		for (int i = 0; i < 3; i++)
		{
			xs[i] = int(floor(v[i].x * 4.0 + 0.5));
			ys[i] = int(floor(v[i].y * 4.0 + 0.5));
		}
		int order[3] = { 0, 1, 2 };
		std::sort(order, order + 3, [&](int a, int b) { return ys[a] != ys[b] ? ys[a] < ys[b] : xs[a] < xs[b]; });
		int i0 = order[0], i1 = order[1], i2 = order[2];
		int y0 = ys[i0], y1 = ys[i1], y2 = ys[i2];
		int x0 = xs[i0], x1 = xs[i1], x2 = xs[i2];
		if (y2 == y0) return false;
		long long cross = (long long)(x2 - x0) * (y1 - y0) - (long long)(y2 - y0) * (x1 - x0);
		if (cross == 0) return false;
		bool lft = cross < 0;

		// Slopes in pixels per scanline (10.2 units cancel), encoded s15.16.
		double sh = double(x2 - x0) / double(y2 - y0);
		double sm = y1 != y0 ? double(x1 - x0) / double(y1 - y0) : 0.0;
		double sl = y2 != y1 ? double(x2 - x1) / double(y2 - y1) : 0.0;
		int32_t dxhdy = to_fixed16(sh) & ~7, dxmdy = to_fixed16(sm) & ~7, dxldy = to_fixed16(sl) & ~7;
		// xh/xm are the edge positions at the top of the scanline containing yh.
		double top_y = double(y0 & ~3) / 4.0;
		double xh_top = x0 / 4.0 + sh * (top_y - y0 / 4.0);
		double xm_top = x0 / 4.0 + sm * (top_y - y0 / 4.0);
		int32_t xh = to_fixed16(xh_top), xm = to_fixed16(xm_top), xl = to_fixed16(x1 / 4.0);

		uint32_t op = OP_TRI | (shade ? 4 : 0) | (tex ? 2 : 0) | (z ? 1 : 0);
		uint32_t w[44];
		int n = 0;
		w[n++] = (op << 24) | (lft ? 1u << 23 : 0) | ((max_level & 7) << 19) | ((tile & 7) << 16) | (uint32_t(y2) & 0x3fff);
		w[n++] = ((uint32_t(y1) & 0x3fff) << 16) | (uint32_t(y0) & 0x3fff);
		w[n++] = uint32_t(xl);
		w[n++] = uint32_t(dxldy);
		w[n++] = uint32_t(xh);
		w[n++] = uint32_t(dxhdy);
		w[n++] = uint32_t(xm);
		w[n++] = uint32_t(dxmdy);

		// Attribute planes from the three vertices (pixel units).
		double X0 = v[i0].x, Y0 = v[i0].y, X1 = v[i1].x, Y1 = v[i1].y, X2 = v[i2].x, Y2 = v[i2].y;
		double det = (X1 - X0) * (Y2 - Y0) - (X2 - X0) * (Y1 - Y0);
		if (fabs(det) < 1e-9) return false;
		auto plane = [&](double a0, double a1, double a2, double &val, double &ddx, double &dde, double &ddy) {
			ddx = ((a1 - a0) * (Y2 - Y0) - (a2 - a0) * (Y1 - Y0)) / det;
			ddy = ((a2 - a0) * (X1 - X0) - (a1 - a0) * (X2 - X0)) / det;
			dde = ddy + ddx * sh;
			val = a0 + ddx * (xh_top - X0) + ddy * (top_y - Y0);
		};
		if (shade)
		{
			int32_t c[4], dx[4], de[4], dy[4];
			for (int k = 0; k < 4; k++)
			{
				double val, ddx, dde, ddy;
				plane(v[i0].c[k], v[i1].c[k], v[i2].c[k], val, ddx, dde, ddy);
				c[k] = to_fixed16(val);
				dx[k] = to_fixed16(ddx);
				de[k] = to_fixed16(dde);
				dy[k] = to_fixed16(ddy);
			}
			auto pack_hi = [](int32_t a, int32_t b) { return (uint32_t(a) & 0xffff0000u) | (uint32_t(b) >> 16); };
			auto pack_lo = [](int32_t a, int32_t b) { return (uint32_t(a) << 16) | (uint32_t(b) & 0xffffu); };
			w[n + 0] = pack_hi(c[0], c[1]);
			w[n + 1] = pack_hi(c[2], c[3]);
			w[n + 2] = pack_hi(dx[0], dx[1]);
			w[n + 3] = pack_hi(dx[2], dx[3]);
			w[n + 4] = pack_lo(c[0], c[1]);
			w[n + 5] = pack_lo(c[2], c[3]);
			w[n + 6] = pack_lo(dx[0], dx[1]);
			w[n + 7] = pack_lo(dx[2], dx[3]);
			w[n + 8] = pack_hi(de[0], de[1]);
			w[n + 9] = pack_hi(de[2], de[3]);
			w[n + 10] = pack_hi(dy[0], dy[1]);
			w[n + 11] = pack_hi(dy[2], dy[3]);
			w[n + 12] = pack_lo(de[0], de[1]);
			w[n + 13] = pack_lo(de[2], de[3]);
			w[n + 14] = pack_lo(dy[0], dy[1]);
			w[n + 15] = pack_lo(dy[2], dy[3]);
			n += 16;
		}
		if (tex)
		{
			int32_t c[3], dx[3], de[3], dy[3];
			double a[3][3] = { { v[i0].s, v[i1].s, v[i2].s }, { v[i0].t, v[i1].t, v[i2].t },
			                   { v[i0].w * 32767.0, v[i1].w * 32767.0, v[i2].w * 32767.0 } };
			for (int k = 0; k < 3; k++)
			{
				double val, ddx, dde, ddy;
				plane(a[k][0], a[k][1], a[k][2], val, ddx, dde, ddy);
				c[k] = to_fixed16(val);
				dx[k] = to_fixed16(ddx);
				de[k] = to_fixed16(dde);
				dy[k] = to_fixed16(ddy);
			}
			auto pack_hi = [](int32_t a, int32_t b) { return (uint32_t(a) & 0xffff0000u) | (uint32_t(b) >> 16); };
			auto pack_lo = [](int32_t a, int32_t b) { return (uint32_t(a) << 16) | (uint32_t(b) & 0xffffu); };
			w[n + 0] = pack_hi(c[0], c[1]);
			w[n + 1] = pack_hi(c[2], 0);
			w[n + 2] = pack_hi(dx[0], dx[1]);
			w[n + 3] = pack_hi(dx[2], 0);
			w[n + 4] = pack_lo(c[0], c[1]);
			w[n + 5] = pack_lo(c[2], 0);
			w[n + 6] = pack_lo(dx[0], dx[1]);
			w[n + 7] = pack_lo(dx[2], 0);
			w[n + 8] = pack_hi(de[0], de[1]);
			w[n + 9] = pack_hi(de[2], 0);
			w[n + 10] = pack_hi(dy[0], dy[1]);
			w[n + 11] = pack_hi(dy[2], 0);
			w[n + 12] = pack_lo(de[0], de[1]);
			w[n + 13] = pack_lo(de[2], 0);
			w[n + 14] = pack_lo(dy[0], dy[1]);
			w[n + 15] = pack_lo(dy[2], 0);
			n += 16;
		}
		if (z)
		{
			double val, ddx, dde, ddy;
			plane(v[i0].z, v[i1].z, v[i2].z, val, ddx, dde, ddy);
			w[n++] = uint32_t(to_fixed16(val));
			w[n++] = uint32_t(to_fixed16(ddx));
			w[n++] = uint32_t(to_fixed16(dde));
			w[n++] = uint32_t(to_fixed16(ddy));
		}
		emit(w, n);
		prims++;
		return true;
	}

	// A random triangle: centroid uniform over the screen, log-normal area.
	void random_triangle_geometry(Vertex v[3])
	{
		double area = p.area_median * Rng::det_exp(p.area_sigma * rng.normal());
		area = std::min(area, double(p.width) * double(p.height));
		const double span_x = (p.flags & RDPGEN_HOTSPOT) ? 16.0 : double(p.width);
		const double span_y = (p.flags & RDPGEN_HOTSPOT) ? 16.0 : double(p.height);
		double cx = rng.uniform() * span_x, cy = rng.uniform() * span_y;
		double px[3], py[3];
		double a = 0;
		for (int tries = 0; tries < 8; tries++)
		{
			for (int i = 0; i < 3; i++)
			{
				double ang = rng.uniform() * 6.283185307179586;
				double r = 0.3 + 0.7 * rng.uniform();
				px[i] = Rng::det_cos(ang) * r;
				py[i] = Rng::det_cos(ang - 1.5707963267948966) * r;
			}
			a = 0.5 * fabs((px[1] - px[0]) * (py[2] - py[0]) - (px[2] - px[0]) * (py[1] - py[0]));
			if (a > 0.05) break;
		}
		double scale = sqrt(area / std::max(a, 1e-3));
		for (int i = 0; i < 3; i++)
		{
			v[i].x = std::min(std::max(cx + px[i] * scale, 0.0), double(p.width) - 0.25);
			v[i].y = std::min(std::max(cy + py[i] * scale, 0.0), double(p.height) - 0.25);
		}
	}

	void random_colors(Vertex v[3])
	{
		for (int i = 0; i < 3; i++)
		{
			for (int k = 0; k < 4; k++) v[i].c[k] = double(rng.below(256));
			v[i].z = double(rng.below(32768));
		}
	}

	void random_texcoords(Vertex v[3], double tex_size, bool persp)
	{
		double base_s = rng.uniform() * 4 * tex_size, base_t = rng.uniform() * 4 * tex_size;
		double scale = 0.25 + rng.uniform() * 2.0;
		for (int i = 0; i < 3; i++)
		{
			double s = (base_s + (v[i].x - v[0].x) * scale) * 32.0;
			double t = (base_t + (v[i].y - v[0].y) * scale) * 32.0;
			double w = persp ? (0.3 + 0.7 * rng.uniform()) : 1.0;
			v[i].w = w;
			v[i].s = std::max(std::min(s * w, 32000.0), -32000.0);
			v[i].t = std::max(std::min(t * w, 32000.0), -32000.0);
		}
	}

	Combiner random_combiner(bool two_cycle)
	{
		Combiner c;
		for (int cy = 0; cy < 2; cy++)
		{
			c.rgb[cy][0] = rng.below(8);    // A: combined..noise
			c.rgb[cy][1] = rng.below(8);    // B: combined..K4
			c.rgb[cy][2] = rng.below(16);   // C: combined..K5
			c.rgb[cy][3] = rng.below(8);    // D: combined..zero
			c.alpha[cy][0] = rng.below(8);
			c.alpha[cy][1] = rng.below(8);
			c.alpha[cy][2] = rng.below(8);
			c.alpha[cy][3] = rng.below(8);
		}
		if (!two_cycle)
		{
			// LOD fraction is only defined in 2-cycle mode (the reference project's README lists reading it in
			// 1-cycle mode as unsupported): keep it out of 1-cycle combiners.
			if (c.rgb[1][2] == 13) c.rgb[1][2] = 4;
			if (c.alpha[1][2] == 0) c.alpha[1][2] = 4;
		}
		return c;
	}

	static Combiner shade_combiner()
	{
		Combiner c;
		for (int cy = 0; cy < 2; cy++)
		{
			c.rgb[cy][0] = 8; c.rgb[cy][1] = 8; c.rgb[cy][2] = 16; c.rgb[cy][3] = 4;   // 0*0 + SHADE
			c.alpha[cy][0] = 7; c.alpha[cy][1] = 7; c.alpha[cy][2] = 7; c.alpha[cy][3] = 4;
		}
		return c;
	}
	static Combiner texture_combiner()
	{
		Combiner c;
		for (int cy = 0; cy < 2; cy++)
		{
			c.rgb[cy][0] = 1; c.rgb[cy][1] = 8; c.rgb[cy][2] = 4; c.rgb[cy][3] = 7;    // TEXEL0 * SHADE
			c.alpha[cy][0] = 1; c.alpha[cy][1] = 7; c.alpha[cy][2] = 4; c.alpha[cy][3] = 7;
		}
		return c;
	}

	uint32_t random_color() { return rng.u32(); }

	// Load an RGBA16 32x32 texture (with its 16x16 and 8x8 mips when lod) into TMEM.
	void load_rgba16_texture(uint32_t slot, bool with_mips, bool random_wrap)
	{
		uint32_t base = TEX_ADDR + slot * 0x1000;
		emit2(uint32_t(OP_SYNC_LOAD) << 24, 0);
		set_texture_image(base, 0, 2, 32);
		set_tile(7, 0, 2, 8, 0, 0, 0, 0, 0, 0, 0, 0);
		tile_cmd(OP_LOAD_TILE, 7, 0, 0, 31 << 2, 31 << 2);
		uint32_t cm_s = random_wrap ? rng.below(4) : 0, cm_t = random_wrap ? rng.below(4) : 0;
		uint32_t mk_s = random_wrap ? 3 + rng.below(3) : 5, mk_t = random_wrap ? 3 + rng.below(3) : 5;
		set_tile(0, 0, 2, 8, 0, 0, cm_t, mk_t, 0, cm_s, mk_s, 0);
		tile_cmd(OP_SET_TILE_SIZE, 0, 0, 0, 31 << 2, 31 << 2);
		if (with_mips)
		{
			// 16x16 at TMEM 2048 B (qw 256), 8x8 at 2560 B (qw 320): loaded as 16-bit lines from the blob.
			set_texture_image(base + 2048, 0, 2, 16);
			set_tile(7, 0, 2, 4, 256, 0, 0, 0, 0, 0, 0, 0);
			tile_cmd(OP_LOAD_TILE, 7, 0, 0, 15 << 2, 15 << 2);
			set_texture_image(base + 2048 + 512, 0, 2, 8);
			set_tile(7, 0, 2, 2, 320, 0, 0, 0, 0, 0, 0, 0);
			tile_cmd(OP_LOAD_TILE, 7, 0, 0, 7 << 2, 7 << 2);
			set_tile(1, 0, 2, 4, 256, 0, cm_t, 4, 1, cm_s, 4, 1);
			tile_cmd(OP_SET_TILE_SIZE, 1, 0, 0, 15 << 2, 15 << 2);
			set_tile(2, 0, 2, 2, 320, 0, cm_t, 3, 2, cm_s, 3, 2);
			tile_cmd(OP_SET_TILE_SIZE, 2, 0, 0, 7 << 2, 7 << 2);
		}
		emit2(uint32_t(OP_SYNC_TILE) << 24, 0);
	}

	// Load a CI8 32x32 texture (LoadBlock) plus a 256-entry TLUT into the upper half of TMEM.
	void load_ci8_texture(uint32_t slot)
	{
		uint32_t ci = TEX_ADDR + 0x10000 + slot * 0x400;
		uint32_t lut = TEX_ADDR + 0x20000 + slot * 0x200;
		emit2(uint32_t(OP_SYNC_LOAD) << 24, 0);
		set_texture_image(lut, 0, 2, 1);
		set_tile(7, 0, 0, 0, 256, 0, 0, 0, 0, 0, 0, 0);
		tile_cmd(OP_LOAD_TLUT, 7, 0, 0, 255 << 2, 0);
		// LoadBlock of 1024 bytes as 16-bit words: 512 texels, dxt for a 32-byte (4 qw) line.
		set_texture_image(ci, 2, 2, 1);
		set_tile(7, 2, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0);
		uint32_t dxt = (2048 + 3) / 4;
		tile_cmd(OP_LOAD_BLOCK, 7, 0, 0, 511, dxt);
		uint32_t cm_t0 = rng.below(4);
		uint32_t cm_s0 = rng.below(4);
		set_tile(0, 2, 1, 4, 0, 0, cm_t0, 5, 0, cm_s0, 5, 0);
		tile_cmd(OP_SET_TILE_SIZE, 0, 0, 0, 31 << 2, 31 << 2);
		emit2(uint32_t(OP_SYNC_TILE) << 24, 0);
	}

	void texrect(uint32_t tile, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1, int s, int t, int dsdx, int dtdy)
	{
		uint32_t w[4];
		w[0] = (uint32_t(OP_TEXRECT) << 24) | ((x1 & 0xfff) << 12) | (y1 & 0xfff);
		w[1] = ((tile & 7) << 24) | ((x0 & 0xfff) << 12) | (y0 & 0xfff);
		w[2] = ((uint32_t(s) & 0xffff) << 16) | (uint32_t(t) & 0xffff);
		w[3] = ((uint32_t(dsdx) & 0xffff) << 16) | (uint32_t(dtdy) & 0xffff);
		emit(w, 4);
		prims++;
	}

	// ------------------------------------------------------------------ frames
	void frame_prologue(uint32_t frame)
	{
		frame_begin.push_back(uint32_t(words.size()));
		set_color_image(COLOR_ADDR, fb_size_bits(), p.width, fb_fmt_bits());
		emit2(uint32_t(OP_SET_MASK_IMAGE) << 24, DEPTH_ADDR);
		set_scissor(p.width, p.height);
		if (p.flags & RDPGEN_CLEAR)
		{
			OtherModes fill;
			fill.cycle = 3;
			set_other_modes(fill);
			uint32_t col = p.fb_format == RDPGEN_FB_RGBA8888 ? random_color() : ((rng.u32() & 0xfffe) * 0x10001u);
			color_reg(OP_SET_FILL_COLOR, col);
			fill_rect(0, 0, (p.width - 1) << 2, (p.height - 1) << 2);
			prims++;
			if (p.flags & (RDPGEN_Z | RDPGEN_Z_HALF))
			{
				// Clear the depth buffer to the far plane through a 16-bit colour image.
				set_color_image(DEPTH_ADDR, 2, p.width);
				color_reg(OP_SET_FILL_COLOR, 0xfffcfffcu);
				fill_rect(0, 0, (p.width - 1) << 2, (p.height - 1) << 2);
				prims++;
				set_color_image(COLOR_ADDR, fb_size_bits(), p.width, fb_fmt_bits());
			}
		}
		(void)frame;
	}

	OtherModes base_modes() const
	{
		OtherModes om;
		om.cycle = (p.flags & RDPGEN_2CYCLE) ? 1 : 0;
		om.persp = (p.flags & RDPGEN_PERSPECTIVE) != 0;
		om.aa = (p.flags & RDPGEN_AA) != 0;
		om.rgb_dither = (p.flags & RDPGEN_DITHER) ? 0 : 3;
		om.alpha_dither = 3;
		om.sample_quad = (p.flags & RDPGEN_BILINEAR) != 0;
		om.bilerp0 = om.bilerp1 = true;
		if (p.flags & RDPGEN_FOG)
		{
			// Cycle 0: fog blend (FOG * shade alpha + pixel * (1 - a)); cycle 1: pixel/memory AA blend.
			om.blend[0][0] = 3; om.blend[0][1] = 2; om.blend[0][2] = 0; om.blend[0][3] = 0;
			om.blend[1][0] = 0; om.blend[1][1] = 0; om.blend[1][2] = 1; om.blend[1][3] = 0;
		}
		if (om.aa) { om.image_read = true; om.cvg_mode = 0; }
		if (p.flags & RDPGEN_Z) { om.z_compare = om.z_update = true; }
		return om;
	}

	// ------------------------------------------------------------------ fuzz streams
	// Random everything, in the spirit of the reference's conformance generator
	// (rdp_conformance.cpp:283-607): each primitive draws its own other-modes bits,
	// combiner and blender selectors, texture format, tile parameters and load method.
	static constexpr uint32_t FUZZ_BLOB = TEX_ADDR + 0x40000;

	void fuzz_texture()
	{
		static const uint32_t kinds[][2] = { { 0, 2 }, { 0, 3 }, { 3, 0 }, { 3, 1 }, { 3, 2 }, { 4, 0 }, { 4, 1 },
		                                     { 2, 0 }, { 2, 1 }, { 1, 2 }, { 0, 1 }, { 2, 2 } };
		const uint32_t *k = kinds[rng.below(12)];
		uint32_t fmt = k[0], siz = k[1];
		uint32_t w = 4u << rng.below(4), h = 4u << rng.below(4);
		uint32_t bits = 4u << siz;
		uint32_t row_bytes = std::max(8u, (w * bits) / 8);
		while (row_bytes * h > (siz == 3 || fmt == 1 ? 2048u : 4096u) && h > 1) h >>= 1;
		uint32_t blob_index = rng.below(8);
		uint32_t blob_offset = rng.below(4) << 3;
		uint32_t blob = FUZZ_BLOB + blob_index * 0x1000 + blob_offset;
		// Sometimes load from an image this stream renders into (a read-after-write hazard).
		uint32_t rt = rng.below(16);
		if (rt == 0) blob = COLOR_ADDR + (rng.below(64) << 6);
		else if (rt == 1) blob = LAYER_ADDR + (rng.below(64) << 6);
		uint32_t line_qw = row_bytes / 8;
		uint32_t tmem_qw = (siz == 3 || fmt == 1) ? rng.below(2) * 8 : rng.below(4) * 16;
		emit2(uint32_t(OP_SYNC_LOAD) << 24, 0);
		// 4/8-bit texels are loaded as 16-bit words; 32-bit texels as 32-bit words.
		uint32_t load_size = siz == 3 ? 3 : 2;
		uint32_t load_texels_per_row = row_bytes / (load_size == 3 ? 4 : 2);
		set_texture_image(blob, fmt, load_size, load_texels_per_row);
		set_tile(7, fmt, load_size, line_qw, tmem_qw, 0, 0, 0, 0, 0, 0, 0);
		uint32_t method = rng.below(3);
		if (method == 0 || siz == 3 || fmt == 1)
			tile_cmd(OP_LOAD_TILE, 7, 0, 0, (load_texels_per_row - 1) << 2, (h - 1) << 2);
		else
		{
			uint32_t texels = load_texels_per_row * h;
			uint32_t dxt = (2048 + line_qw - 1) / line_qw;
			if (method == 2) set_tile(7, fmt, load_size, 0, tmem_qw, 0, 0, 0, 0, 0, 0, 0);
			tile_cmd(OP_LOAD_BLOCK, 7, 0, 0, std::min(texels, 2048u) - 1, dxt);
		}
		if (fmt == 2 || (rng.u32() & 3) == 0)
		{
			// TLUT: 16 or 256 entries into the upper half of TMEM.
			uint32_t entries = (siz == 0 && (rng.u32() & 1)) ? 16 : 256;
			uint32_t lut_tmem = 256 + (entries == 16 ? rng.below(16) * 16 : 0);
			set_texture_image(TEX_ADDR + 0x20000 + rng.below(NUM_TEX) * 0x200, 0, 2, 1);
			set_tile(7, 0, 0, 0, lut_tmem, 0, 0, 0, 0, 0, 0, 0);
			tile_cmd(OP_LOAD_TLUT, 7, 0, 0, (entries - 1) << 2, 0);
		}
		uint32_t cm_s = rng.below(4), cm_t = rng.below(4);
		uint32_t mk_s = rng.below(6), mk_t = rng.below(6);
		uint32_t sh_s = rng.below(4) == 0 ? rng.below(16) : 0, sh_t = rng.below(4) == 0 ? rng.below(16) : 0;
		for (uint32_t t = 0; t < 3; t++)
		{
			set_tile(t, fmt, siz, line_qw >> (t ? 1 : 0), tmem_qw + t * 32, rng.below(16), cm_t, mk_t, sh_t, cm_s, mk_s, sh_s);
			uint32_t sl = rng.below(3) == 0 ? rng.below(16) : 0, tl = rng.below(3) == 0 ? rng.below(16) : 0;
			uint32_t sh_frac = rng.below(4);
			uint32_t th_frac = rng.below(4);
			tile_cmd(OP_SET_TILE_SIZE, t, sl, tl, sl + ((w - 1) << 2) + sh_frac, tl + ((h - 1) << 2) + th_frac);
		}
		emit2(uint32_t(OP_SYNC_TILE) << 24, 0);
	}

	OtherModes fuzz_modes(uint32_t cycle)
	{
		OtherModes m;
		m.cycle = cycle;
		m.persp = rng.u32() & 1;
		m.detail = (rng.u32() & 3) == 0;
		m.sharpen = (rng.u32() & 3) == 0;
		m.tex_lod = (rng.u32() & 3) == 0;
		m.tlut = (rng.u32() & 3) == 0;
		m.tlut_ia = rng.u32() & 1;
		m.sample_quad = rng.u32() & 1;
		m.mid_texel = (rng.u32() & 3) == 0;
		m.bilerp0 = rng.u32() & 1;
		m.bilerp1 = rng.u32() & 1;
		m.convert_one = (rng.u32() & 3) == 0;
		m.rgb_dither = rng.below(4);
		m.alpha_dither = rng.below(4);
		for (int c = 0; c < 2; c++)
			for (int i = 0; i < 4; i++) m.blend[c][i] = rng.below(4);
		m.force_blend = rng.u32() & 1;
		m.alpha_cvg_select = (rng.u32() & 3) == 0;
		m.cvg_times_alpha = (rng.u32() & 3) == 0;
		m.z_mode = rng.below(4);
		m.cvg_mode = rng.below(4);
		m.color_on_cvg = (rng.u32() & 3) == 0;
		m.image_read = rng.u32() & 1;
		m.z_compare = rng.u32() & 1;
		m.z_update = rng.u32() & 1;
		m.aa = rng.u32() & 1;
		m.prim_depth = (rng.u32() & 7) == 0;
		m.alpha_test = (rng.u32() & 3) == 0;
		m.alpha_test_dither = (rng.u32() & 3) == 0;
		return m;
	}

	void build_fuzz()
	{
		make_textures();
		for (uint32_t k = 0; k < 8; k++)
		{
			Blob b;
			b.addr = FUZZ_BLOB + k * 0x1000;
			b.bytes.resize(0x1000 + 64);
			for (auto &v : b.bytes) v = uint8_t(rng.u32());
			blobs.push_back(std::move(b));
		}
		for (uint32_t f = 0; f < std::max(1u, p.num_frames); f++)
		{
			frame_prologue(f);
			set_color_image(COLOR_ADDR, fb_size_bits(), p.width, fb_fmt_bits());
			uint32_t emitted = 0;
			while (emitted < p.num_prims)
			{
				uint32_t r = rng.below(100);
				if (r < 3)
				{
					// Random scissor, sometimes interlaced.
					uint32_t x0 = rng.below(p.width / 2), y0 = rng.below(p.height / 2);
					uint32_t x1 = p.width / 2 + rng.below(p.width / 2 + 1), y1 = p.height / 2 + rng.below(p.height / 2 + 1);
					uint32_t il = (rng.u32() & 3) == 0 ? (2u | (rng.u32() & 1)) : 0;
					uint32_t f[4];
					for (auto &v : f) v = rng.below(4);
					emit2((uint32_t(OP_SET_SCISSOR) << 24) | (((x0 << 2) + f[0]) << 12) | ((y0 << 2) + f[1]),
					      (il << 24) | (((x1 << 2) - f[2]) << 12) | ((y1 << 2) - f[3]));
				}
				if (r < 12) fuzz_texture();
				if (r >= 96)
				{
					// Switch the colour image: the main image, or a second image at LAYER_ADDR in
					// a random format and width (several images per pass, I8 among them).
					uint32_t pick = rng.below(3);
					if (pick == 0)
						set_color_image(COLOR_ADDR, fb_size_bits(), p.width, fb_fmt_bits());
					else
					{
						static const uint32_t fmts[][2] = { { 2, 0 }, { 2, 3 }, { 1, 0 }, { 3, 0 }, { 0, 0 } }; // size, fmt bits
						const uint32_t *f = fmts[rng.below(5)];
						uint32_t lw = pick == 1 ? p.width : 64 + rng.below(p.width - 63);
						set_color_image(LAYER_ADDR, f[0], lw, f[1]);
					}
				}
				if (r < 20)
				{
					uint32_t cv0 = rng.u32() & 0x3fffff;
					uint32_t cv1 = rng.u32();
					emit2(uint32_t(OP_SET_CONVERT) << 24 | cv0, cv1);
					emit2(uint32_t(0x2b) << 24, rng.u32() & 0x0fffffff);
					uint32_t ky0 = rng.u32() & 0xffffff;
					uint32_t ky1 = rng.u32();
					emit2(uint32_t(0x2a) << 24 | ky0, ky1);
					emit2(uint32_t(OP_SET_PRIM_DEPTH) << 24, rng.u32());
					color_reg(OP_SET_FOG_COLOR, rng.u32());
					color_reg(OP_SET_BLEND_COLOR, rng.u32());
				}
				uint32_t kind = rng.below(10);
				bool fill_ok = p.fb_format != RDPGEN_FB_I4;
				uint32_t cycle = rng.below(2);
				if (kind == 8 && fill_ok) cycle = 3;
				if (kind == 9) cycle = 2;
				OtherModes m = fuzz_modes(cycle);
				if (cycle == 3) { m.z_compare = false; m.image_read = false; m.z_update = false; }
				set_other_modes(m);
				set_combiner(random_combiner(cycle == 1));
				uint32_t pc_level = rng.below(32) << 8;
				uint32_t pc_frac = rng.below(256);
				uint32_t pc_color = rng.u32();
				emit2((uint32_t(OP_SET_PRIM_COLOR) << 24) | pc_level | pc_frac, pc_color);
				color_reg(OP_SET_ENV_COLOR, rng.u32());
				if (cycle == 3) color_reg(OP_SET_FILL_COLOR, rng.u32());
				if (kind < 6 || (kind == 8 && !fill_ok))
				{
					Vertex v[3];
					random_triangle_geometry(v);
					random_colors(v);
					random_texcoords(v, 32.0, m.persp);
					bool shade = rng.u32() & 1, tex = rng.u32() & 1, z = rng.u32() & 1;
					uint32_t tri_tile = rng.below(8);
					uint32_t tri_level = rng.below(8);
					if (emit_triangle(v, shade, tex, z, tri_tile, tri_level)) emitted++;
				}
				else if (kind == 8)
				{
					uint32_t w = 1 + rng.below(48), h = 1 + rng.below(48);
					uint32_t x0 = rng.below(p.width), y0 = rng.below(p.height);
					uint32_t q[4];
					for (auto &v : q) v = rng.below(4);
					fill_rect((x0 << 2) + q[0], (y0 << 2) + q[1], ((x0 + w) << 2) + q[2], ((y0 + h) << 2) + q[3]);
					prims++;
					emitted++;
				}
				else
				{
					uint32_t w = 1 + rng.below(40), h = 1 + rng.below(40);
					uint32_t x0 = rng.below(p.width), y0 = rng.below(p.height);
					int dsdx = cycle == 2 ? (4 << 10) : int(rng.below(0x1000)) - 0x800;
					int dtdy = int(rng.below(0x1000)) - 0x400;
					uint32_t wq[4];
					uint32_t op = (rng.u32() & 1) ? OP_TEXRECT : (OP_TEXRECT + 1);
					uint32_t q[8];
					for (auto &v : q) v = rng.below(4);
					uint32_t rect_tile = rng.below(8);
					uint32_t s16 = rng.u32() & 0xffffu;
					uint32_t t16 = rng.u32() & 0xffffu;
					wq[0] = (op << 24) | ((((x0 + w) << 2) + q[0]) << 12) | (((y0 + h) << 2) + q[1]);
					wq[1] = (rect_tile << 24) | (((x0 << 2) + q[2]) << 12) | ((y0 << 2) + q[3]);
					wq[2] = s16 << 16 | t16;
					wq[3] = ((uint32_t(dsdx) & 0xffff) << 16) | (uint32_t(dtdy) & 0xffff);
					emit(wq, 4);
					prims++;
					emitted++;
				}
			}
			emit2(uint32_t(OP_SYNC_FULL) << 24, 0);
		}
	}

	void build()
	{
		if (p.flags & RDPGEN_FUZZ)
		{
			build_fuzz();
			return;
		}
		make_textures();
		Rng mixrng(uint64_t(p.seed) * 7919 + 3);
		uint32_t weights[5] = { p.w_shade_tri, p.w_tex_tri, p.w_copy_rect, p.w_ci8_tri, p.w_fill_rect };
		uint32_t wsum = 0;
		for (auto w : weights) wsum += w;
		if (!wsum) { weights[0] = 1; wsum = 1; }

		for (uint32_t f = 0; f < std::max(1u, p.num_frames); f++)
		{
			frame_prologue(f);
			color_reg(OP_SET_FOG_COLOR, random_color());
			color_reg(OP_SET_BLEND_COLOR, random_color() & 0xffffff00u);
			color_reg(OP_SET_ENV_COLOR, random_color());
			emit2((uint32_t(OP_SET_PRIM_COLOR) << 24), random_color());
			int current_kind = -1;
			uint32_t run_left = 0, tex_left = 0;
			bool layer_bound = false, run_lod = false;
			uint32_t frame_target = p.num_prims;
			uint32_t emitted = 0;
			uint32_t last_modes[2] = { 0, 0 }, last_comb[2] = { 0, 0 };
			auto modes = [&](const OtherModes &m) {
				uint32_t w[2];
				m.encode(w);
				if (w[0] != last_modes[0] || w[1] != last_modes[1]) { emit(w, 2); last_modes[0] = w[0]; last_modes[1] = w[1]; }
			};
			auto comb = [&](const Combiner &c) {
				uint32_t w[2];
				c.encode(w);
				if (w[0] != last_comb[0] || w[1] != last_comb[1]) { emit(w, 2); last_comb[0] = w[0]; last_comb[1] = w[1]; }
			};
			while (emitted < frame_target)
			{
				if (run_left == 0)
				{
					int prev_kind = current_kind;
					uint32_t r = mixrng.below(wsum), acc = 0;
					for (int k = 0; k < 5; k++)
					{
						acc += weights[k];
						if (r < acc) { current_kind = k; break; }
					}
					if (current_kind != prev_kind) tex_left = 0;
					run_left = (p.flags & RDPGEN_RUNS) ? 16 + mixrng.below(96) : 1;
					// Copy mode writes nothing on a 32-bit colour image (memory_interfacing.h:381-420), so
					// copy-mode rectangles of a 32-bit frame go to a 16-bit layer image.
					bool want_layer = current_kind == 2 && p.fb_format == RDPGEN_FB_RGBA8888;
					if (want_layer != layer_bound)
					{
						if (want_layer) set_color_image(LAYER_ADDR, 2, p.width);
						else set_color_image(COLOR_ADDR, fb_size_bits(), p.width);
						layer_bound = want_layer;
					}
				}
				run_left--;
				bool zprim = (p.flags & RDPGEN_Z) || ((p.flags & RDPGEN_Z_HALF) && (rng.u32() & 1));
				bool atest = (p.flags & RDPGEN_ALPHA_TEST_HALF) && (rng.u32() & 1);
				switch (current_kind)
				{
				case 0: // Gouraud triangle
				{
					OtherModes m = base_modes();
					m.z_compare = m.z_update = zprim;
					m.alpha_test = atest;
					if (p.flags & RDPGEN_RANDOM_COMBINER)
					{
						comb(random_combiner(m.cycle == 1));
						uint32_t lod_frac = rng.below(256);
						emit2((uint32_t(OP_SET_PRIM_COLOR) << 24) | lod_frac, random_color());
						color_reg(OP_SET_ENV_COLOR, random_color());
					}
					else
						comb(shade_combiner());
					modes(m);
					Vertex v[3];
					random_triangle_geometry(v);
					random_colors(v);
					if (emit_triangle(v, true, false, zprim, 0, 0)) emitted++;
					break;
				}
				case 1: // textured triangle, RGBA16
				case 3: // CI8 + TLUT
				{
					bool ci = current_kind == 3;
					if (tex_left == 0)
					{
						run_lod = (p.flags & RDPGEN_LOD) && !ci && (rng.u32() & 1);
						if (ci) load_ci8_texture(rng.below(NUM_TEX));
						else load_rgba16_texture(rng.below(NUM_TEX), run_lod, true);
						tex_left = 4 + rng.below(13);
					}
					tex_left--;
					bool lod = run_lod && (rng.u32() & 1);
					OtherModes m = base_modes();
					m.z_compare = m.z_update = zprim;
					m.alpha_test = atest;
					m.tlut = ci;
					m.sample_quad = (p.flags & RDPGEN_BILINEAR) != 0;
					if (lod)
					{
						m.cycle = 1;
						m.tex_lod = true;
						m.detail = (rng.u32() & 3) == 0;
					}
					modes(m);
					if (p.flags & RDPGEN_RANDOM_COMBINER)
					{
						comb(random_combiner(m.cycle == 1));
						uint32_t lod_frac = rng.below(256);
						uint32_t min_level = rng.below(3) << 8;
						emit2((uint32_t(OP_SET_PRIM_COLOR) << 24) | lod_frac | min_level, random_color());
						color_reg(OP_SET_ENV_COLOR, random_color());
					}
					else
						comb(texture_combiner());
					Vertex v[3];
					random_triangle_geometry(v);
					random_colors(v);
					random_texcoords(v, 32.0, (p.flags & RDPGEN_PERSPECTIVE) != 0);
					if (emit_triangle(v, true, true, zprim, 0, lod ? 2 : 0)) emitted++;
					break;
				}
				case 2: // TextureRectangle in copy mode
				{
					if (tex_left == 0)
					{
						load_rgba16_texture(rng.below(NUM_TEX), false, false);
						tex_left = 4 + rng.below(13);
					}
					tex_left--;
					OtherModes m;
					m.cycle = 2;
					m.alpha_test = atest;
					modes(m);
					uint32_t w = 8 + rng.below(48), h = 8 + rng.below(48);
					uint32_t x0 = rng.below(p.width > w ? p.width - w : 1), y0 = rng.below(p.height > h ? p.height - h : 1);
					int s0 = int(rng.below(32)) << 5;
					int t0 = int(rng.below(32)) << 5;
					texrect(0, x0 << 2, y0 << 2, (x0 + w) << 2, (y0 + h) << 2, s0, t0, 4 << 10, 1 << 10);
					emitted++;
					break;
				}
				default: // FillRect
				{
					OtherModes m;
					m.cycle = 3;
					modes(m);
					uint32_t col = p.fb_format == RDPGEN_FB_RGBA8888 && !layer_bound ? random_color()
					                                                               : ((rng.u32() & 0xffff) * 0x10001u);
					color_reg(OP_SET_FILL_COLOR, col);
					uint32_t w = 4 + rng.below(64), h = 4 + rng.below(64);
					uint32_t x0 = rng.below(p.width > w ? p.width - w : 1), y0 = rng.below(p.height > h ? p.height - h : 1);
					fill_rect(x0 << 2, y0 << 2, (x0 + w) << 2, (y0 + h) << 2);
					prims++;
					emitted++;
					break;
				}
				}
			}
			if (layer_bound) set_color_image(COLOR_ADDR, fb_size_bits(), p.width);
			emit2(uint32_t(OP_SYNC_FULL) << 24, 0);
		}
	}
};

} // namespace

extern "C" {

void rdpgen_default_params(rdpgen_params *p, int config)
{
	memset(p, 0, sizeof(*p));
	p->rdram_size = 8u << 20;
	p->num_frames = 1;
	p->area_sigma = 1.5f;
	switch (config)
	{
	case 0: // plain single frame
		p->width = 320; p->height = 240; p->fb_format = RDPGEN_FB_RGBA5551;
		p->num_prims = 2000; p->area_median = 64.0f; p->w_shade_tri = 1;
		p->flags = RDPGEN_CLEAR;
		break;
	case 1: // textured, depth-tested
		p->width = 320; p->height = 240; p->fb_format = RDPGEN_FB_RGBA5551;
		p->num_prims = 10000; p->area_median = 48.0f; p->w_tex_tri = 1;
		p->flags = RDPGEN_CLEAR | RDPGEN_Z | RDPGEN_2CYCLE | RDPGEN_PERSPECTIVE | RDPGEN_BILINEAR | RDPGEN_AA |
		           RDPGEN_DITHER | RDPGEN_FOG | RDPGEN_RANDOM_COMBINER;
		break;
	case 2: // mixed 640x480 RGBA8888 sequence
	default:
		p->width = 640; p->height = 480; p->fb_format = RDPGEN_FB_RGBA8888;
		p->num_prims = 50000; p->num_frames = 16; p->area_median = 48.0f;
		p->w_tex_tri = 40; p->w_copy_rect = 30; p->w_ci8_tri = 20; p->w_fill_rect = 10;
		p->flags = RDPGEN_CLEAR | RDPGEN_Z_HALF | RDPGEN_ALPHA_TEST_HALF | RDPGEN_LOD | RDPGEN_BILINEAR |
		           RDPGEN_PERSPECTIVE | RDPGEN_RUNS;
		break;
	}
}

void *rdpgen_build(const rdpgen_params *params)
{
	Gen *g = new Gen(*params);
	g->build();
	return g;
}

void rdpgen_destroy(void *h) { delete static_cast<Gen *>(h); }
uint32_t rdpgen_num_words(void *h) { return uint32_t(static_cast<Gen *>(h)->words.size()); }
const uint32_t *rdpgen_words(void *h) { return static_cast<Gen *>(h)->words.data(); }
uint32_t rdpgen_num_prims(void *h) { return static_cast<Gen *>(h)->prims; }
uint32_t rdpgen_num_frames(void *h) { return uint32_t(static_cast<Gen *>(h)->frame_begin.size()); }
uint32_t rdpgen_frame_word_offset(void *h, uint32_t frame)
{
	const Gen *g = static_cast<Gen *>(h);
	return frame < g->frame_begin.size() ? g->frame_begin[frame] : uint32_t(g->words.size());
}

void rdpgen_init_rdram(void *h, uint8_t *rdram, uint32_t size)
{
	Gen *g = static_cast<Gen *>(h);
	for (auto &b : g->blobs)
	{
		// RDRAM is stored as host-order 32-bit words; byte address a lives at a ^ 3.
		for (size_t i = 0; i < b.bytes.size(); i++)
		{
			uint32_t a = uint32_t(b.addr + i);
			if (a < size) rdram[a ^ 3] = b.bytes[i];
		}
	}
}

uint32_t rdpgen_color_addr(void) { return Gen::COLOR_ADDR; }
uint32_t rdpgen_depth_addr(void) { return Gen::DEPTH_ADDR; }
}
