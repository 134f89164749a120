/*
 * GB300 (sm_103a) kernels for the N64 RDP rendering path.
 *
 *   k_prim_setup : one thread per primitive.  Decodes the RDP command words and
 *                  the raw state-register block into edge coefficients,
 *                  attributes, derived combiner constants and normalised static
 *                  state (rdp_device.cpp:268-864, rdp_renderer.cpp:717-1562).
 *   k_bin        : one warp per primitive.  Conservative 8x8-tile binning
 *                  (shaders/binning.h) into per-tile primitive bitmasks and counts.
 *   k_span       : one warp per primitive.  The spans of its scanlines
 *                  (shaders/span_setup.comp), once for all its tiles.
 *   k_tmem_*     : TMEM uploads (shaders/tmem_update.comp), one snapshot per upload.
 *   k_scan_*     : pair offsets per tile (and per primitive), control words.
 *   k_expand     : the (primitive, tile) pair list, in primitive order per tile.
 *   k_shade_*    : per-pixel shading of every pair (shaders/shading.h) into scratch,
 *                  pairs in parallel, the pixels a pair can cover packed into warps.
 *   k_blend      : per tile, the pairs' shaded pixels in primitive order through
 *                  depth test, blender, dither and coverage against the tile's
 *                  colour/depth held in registers (shaders/memory_interfacing.h,
 *                  depth_blend.comp); writes back only what was written.
 *   k_raster     : fused shading + blending per tile, taken only when a launch's
 *                  pairs or span rows overflow the scratch.
 *
 * All arithmetic is the RDP's integer fixed point; wrap-around is explicit
 * (unsigned multiplies/shifts) so that it matches 32-bit GLSL semantics.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <stdint.h>
#include "rdp_types.h"
#include "rdp_kernels.h"
#include "sched.h"

namespace rdp {

// ============================================================================ small helpers
__device__ __forceinline__ int mulw(int a, int b) { return int(unsigned(a) * unsigned(b)); }
__device__ __forceinline__ int shlw(int a, int s) { return int(unsigned(a) << s); }
__device__ __forceinline__ int bfe_s(int v, int bits) { return int(unsigned(v) << (32 - bits)) >> (32 - bits); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }
__device__ __forceinline__ int find_msb(int v)
{
	if (v < 0) v = ~v;
	return v ? 31 - __clz(v) : -1;
}
__device__ __forceinline__ int find_lsb(unsigned v) { return v ? __ffs(v) - 1 : -1; }

// Hardware tables: blender divider (luts.hpp:7, regenerated in rdp_luts.cpp),
// magic-square/Bayer dither (dither.h:28-30), perspective reciprocal (perspective.h:27-44).
__device__ uint8_t g_blender_lut[0x8000];

__device__ const uint8_t g_dither[2][16] = {
	{ 0, 6, 1, 7, 4, 2, 5, 3, 3, 5, 2, 4, 7, 1, 6, 0 },
	{ 0, 4, 1, 5, 4, 0, 5, 1, 3, 7, 2, 6, 7, 3, 6, 2 },
};

__device__ const int16_t g_persp_base[64] = {
	0x4000, 0x3f04, 0x3e10, 0x3d22, 0x3c3c, 0x3b5d, 0x3a83, 0x39b1, 0x38e4, 0x381c, 0x375a, 0x369d, 0x35e5, 0x3532, 0x3483, 0x33d9,
	0x3333, 0x3291, 0x31f4, 0x3159, 0x30c3, 0x3030, 0x2fa1, 0x2f15, 0x2e8c, 0x2e06, 0x2d83, 0x2d03, 0x2c86, 0x2c0b, 0x2b93, 0x2b1e,
	0x2aab, 0x2a3a, 0x29cc, 0x2960, 0x28f6, 0x288e, 0x2828, 0x27c4, 0x2762, 0x2702, 0x26a4, 0x2648, 0x25ed, 0x2594, 0x253d, 0x24e7,
	0x2492, 0x243f, 0x23ee, 0x239e, 0x234f, 0x2302, 0x22b6, 0x226c, 0x2222, 0x21da, 0x2193, 0x214d, 0x2108, 0x20c5, 0x2082, 0x2041,
};
__device__ const int16_t g_persp_slope[64] = {
	252, 244, 238, 230, 223, 218, 210, 205, 200, 194, 189, 184, 179, 175, 170, 166,
	162, 157, 155, 150, 147, 143, 140, 137, 134, 131, 128, 125, 123, 120, 117, 115,
	113, 110, 108, 106, 104, 102, 100, 98, 96, 94, 92, 91, 89, 87, 86, 85,
	83, 81, 80, 79, 77, 76, 74, 74, 72, 71, 70, 69, 67, 67, 65, 65,
};

// ============================================================================ k_prim_setup
__device__ __forceinline__ uint32_t merge_hi(uint32_t hi_word, uint32_t lo_word)
{
	return (hi_word & 0xffff0000u) | ((lo_word >> 16) & 0xffffu);
}
__device__ __forceinline__ uint32_t merge_lo(uint32_t hi_word, uint32_t lo_word)
{
	return (hi_word << 16) | (lo_word & 0xffffu);
}

__device__ int norm_muladd(int v) { return (v == 7 || v == 1 || v == 2 || v == 0 || v == 6 || v == 4) ? v : 8; }
__device__ int norm_mulsub(int v) { return (v == 0 || v == 1 || v == 2 || v == 4 || v == 7) ? v : 8; }
__device__ int norm_mul(int v)
{
	return (v == 0 || v == 7 || v == 1 || v == 2 || v == 8 || v == 9 || v == 4 || v == 11 || v == 13 || v == 15) ? v : 16;
}
__device__ int norm_add(int v) { return (v == 1 || v == 2 || v == 0 || v == 6 || v == 4) ? v : 7; }
__device__ int norm_aaddsub(int v) { return (v == 0 || v == 1 || v == 2 || v == 4 || v == 6) ? v : 7; }
__device__ int norm_amul(int v) { return (v == 0 || v == 1 || v == 2 || v == 4) ? v : 7; }

__device__ bool acc_t0(const int rgb[4], const int a[4])
{
	return rgb[0] == 1 || rgb[1] == 1 || rgb[2] == 1 || rgb[3] == 1 || rgb[2] == 8 || a[0] == 1 || a[1] == 1 ||
	       a[2] == 1 || a[3] == 1;
}
__device__ bool acc_t1(const int rgb[4], const int a[4])
{
	return rgb[0] == 2 || rgb[1] == 2 || rgb[2] == 2 || rgb[3] == 2 || rgb[2] == 9 || a[0] == 2 || a[1] == 2 ||
	       a[2] == 2 || a[3] == 2;
}

__device__ void put_rgb(uint8_t *o, uint32_t c)
{
	o[0] = uint8_t(c >> 24);
	o[1] = uint8_t(c >> 16);
	o[2] = uint8_t(c >> 8);
}

// Conservative x range over one y sample (rdp_renderer.cpp:962-992); y is a sub-scanline of the
// image scaled by 2^sl.
__device__ void interp_x64(const RdpPrimGeom &g, int y, bool flip, long long &xl, long long &xr, int sl = 0)
{
	long long yh_base = (long long)(g.yh & ~3) << sl, ym = (long long)g.ym << sl;
	long long xh = ((long long)g.xh << sl) + (long long)(y - yh_base) * g.dxhdy;
	long long xm = ((long long)g.xm << sl) + (long long)(y - yh_base) * g.dxmdy;
	long long xlv = ((long long)g.xl << sl) + (long long)(y - ym) * g.dxldy;
	if (y < ym) xlv = xm;
	long long hs = xh >> 15, ls = xlv >> 15;
	xl = flip ? hs : ls;
	xr = flip ? ls : hs;
	if (xl > 2147483647LL) xl = 2147483647LL;
	if (xl < -2147483648LL) xl = -2147483648LL;
	if (xr > 2147483647LL) xr = 2147483647LL;
	if (xr < -2147483648LL) xr = -2147483648LL;
}

// Pass of a launch that holds primitive i (passes are sorted by their first primitive).
__device__ __forceinline__ uint32_t pass_of_prim(const RdpPass *__restrict__ passes, uint32_t num_passes, uint32_t i)
{
	uint32_t lo = 0, hi = num_passes - 1;
	while (lo < hi)
	{
		uint32_t mid = (lo + hi + 1) >> 1;
		if (passes[mid].prim_begin <= i) lo = mid;
		else hi = mid - 1;
	}
	return lo;
}

// The pass holding tile item `item`, the last with tile_item_begin <= item: a warp's 32 lanes probe
// 32 evenly spaced passes per step (a 32-ary search), two dependent loads for up to 1,024 passes
// where a binary search takes ten.  Called by all lanes of a warp.
__device__ __forceinline__ uint32_t pass_of_item_warp(const RdpPass *__restrict__ passes, uint32_t num_passes,
                                                      uint32_t item, int lane)
{
	// passes[lo].tile_item_begin <= item, and the last such pass lies in [lo, lo + n).
	uint32_t lo = 0, n = num_passes;
	while (n > 1)
	{
		const uint32_t step = (n + 31) / 32;
		const uint32_t cand = lo + uint32_t(lane) * step;
		const bool le = cand < lo + n && passes[cand].tile_item_begin <= item;
		const uint32_t k = 31u - uint32_t(__clz(int(__ballot_sync(0xffffffffu, le))));
		lo += k * step;
		n = min(step, n - k * step);
	}
	return lo;
}

__global__ void k_prim_setup(const RdpPrimIn *__restrict__ in, uint32_t num_prims, const uint32_t *__restrict__ words,
                             const uint32_t *__restrict__ state_blocks, const RdpPass *__restrict__ passes,
                             uint32_t num_passes, RdpPrimGeom *__restrict__ geom_out, RdpPrimAttr *__restrict__ attr_out,
                             RdpPrimShade *__restrict__ shade_out, uint16_t *__restrict__ featbits)
{
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= num_prims) return;
	RdpPrimIn pi = in[i];
	const uint32_t pass_index = pass_of_prim(passes, num_passes, i);
	const RdpPass &pass = passes[pass_index];
	const uint32_t *w = words + pass.word_base + pi.word_offset;
	const uint32_t *sb = state_blocks + size_t(pass.sb_base + pi.state_block) * RDP_STATE_BLOCK_WORDS;

	// ---- other modes (rdp_device.cpp:474-540)
	uint32_t om0 = sb[SB_OTHER_MODES], om1 = sb[SB_OTHER_MODES + 1];
	uint32_t sf = 0, df = 0;
	if (om0 & (1u << 19)) sf |= RS_PERSPECTIVE;
	if (om0 & (1u << 18)) sf |= RS_DETAIL;
	if (om0 & (1u << 17)) sf |= RS_SHARPEN;
	if (om0 & (1u << 16)) sf |= RS_TEX_LOD;
	if (om0 & (1u << 15)) sf |= RS_TLUT;
	if (om0 & (1u << 14)) sf |= RS_TLUT_TYPE;
	if (om0 & (1u << 13)) sf |= RS_SAMPLE_QUAD;
	if (om0 & (1u << 12)) sf |= RS_MID_TEXEL;
	if (om0 & (1u << 11)) sf |= RS_BILERP0;
	if (om0 & (1u << 10)) sf |= RS_BILERP1;
	if (om0 & (1u << 9)) sf |= RS_CONVERT_ONE;
	if (om1 & (1u << 14)) df |= DB_FORCE_BLEND;
	if (om1 & (1u << 13)) sf |= RS_ALPHA_CVG_SELECT;
	if (om1 & (1u << 12)) sf |= RS_CVG_TIMES_ALPHA;
	if (om1 & (1u << 7)) df |= DB_COLOR_ON_CVG;
	if (om1 & (1u << 6)) df |= DB_IMAGE_READ;
	if (om1 & (1u << 5)) df |= DB_DEPTH_UPDATE;
	if (om1 & (1u << 4)) df |= DB_DEPTH_TEST;
	if (om1 & (1u << 3)) { sf |= RS_AA; df |= DB_AA; }
	if (om1 & (1u << 1)) sf |= RS_ALPHA_TEST_DITHER;
	if (om1 & (1u << 0)) sf |= RS_ALPHA_TEST;
	uint32_t dither = (om0 >> 4) & 0xf;
	if ((dither >> 2) != 3) df |= DB_DITHER;
	uint32_t cycle = (om0 >> 20) & 3;
	if (cycle == 1) { sf |= RS_MULTI_CYCLE; df |= DB_MULTI_CYCLE; }
	else if (cycle == 3) sf |= RS_FILL;
	else if (cycle == 2) sf |= RS_COPY;
	bool use_prim_depth = (om1 & (1u << 2)) != 0;

	// ---- combine (rdp_device.cpp:661-684)
	uint32_t c0 = sb[SB_COMBINE], c1 = sb[SB_COMBINE + 1];
	int rgb[2][4], alp[2][4];
	rgb[0][0] = (c0 >> 20) & 0xf; rgb[0][2] = (c0 >> 15) & 0x1f; rgb[0][1] = (c1 >> 28) & 0xf; rgb[0][3] = (c1 >> 15) & 7;
	alp[0][0] = (c0 >> 12) & 7; alp[0][1] = (c1 >> 12) & 7; alp[0][2] = (c0 >> 9) & 7; alp[0][3] = (c1 >> 9) & 7;
	rgb[1][0] = (c0 >> 5) & 0xf; rgb[1][2] = c0 & 0x1f; rgb[1][1] = (c1 >> 24) & 0xf; rgb[1][3] = (c1 >> 6) & 7;
	alp[1][0] = (c1 >> 21) & 7; alp[1][1] = (c1 >> 3) & 7; alp[1][2] = (c1 >> 18) & 7; alp[1][3] = c1 & 7;

	// ---- scissor (rdp_device.cpp:461-472)
	uint32_t s0 = sb[SB_SCISSOR], s1 = sb[SB_SCISSOR + 1];
	RdpPrimGeom g;
	g.scissor[0] = (s0 >> 12) & 0xfff;
	g.scissor[1] = s0 & 0xfff;
	g.scissor[2] = (s1 >> 12) & 0xfff;
	g.scissor[3] = s1 & 0xfff;
	if (s1 & (1u << 25)) sf |= RS_INTERLACE_FIELD;
	if (s1 & (1u << 24)) sf |= RS_INTERLACE_KEEP_ODD;
	uint32_t quirks = sb[SB_QUIRKS];

	// ---- primitive words
	RdpPrimAttr a;
	for (int c = 0; c < 4; c++)
	{
		a.rgba[c] = a.drgba_dx[c] = a.drgba_de[c] = a.drgba_dy[c] = 0;
		a.stzw[c] = a.dstzw_dx[c] = a.dstzw_de[c] = a.dstzw_dy[c] = 0;
	}
	uint32_t op = (w[0] >> 24) & 63;
	uint32_t tflags = 0, tile = 0;
	if (op >= 0x08 && op <= 0x0f)
	{
		// rdp_device.cpp:268-294
		bool flip = (w[0] & 0x800000u) != 0;
		bool sign_dxhdy = (w[5] & 0x80000000u) != 0;
		tflags |= flip ? TRI_FLIP : 0;
		tflags |= (flip == sign_dxhdy) ? TRI_DO_OFFSET : 0;
		tflags |= (sf & RS_COPY) ? TRI_SKIP_XFRAC : 0;
		tflags |= (quirks & 0xff00u) ? TRI_NATIVE_LOD : 0;
		tile = (w[0] >> 16) & 63;
		g.yl = bfe_s(int(w[0]), 14);
		g.ym = bfe_s(int(w[1] >> 16), 14);
		g.yh = bfe_s(int(w[1]), 14);
		g.xl = bfe_s(int(w[2]), 28) >> 1;
		g.xh = bfe_s(int(w[4]), 28) >> 1;
		g.xm = bfe_s(int(w[6]), 28) >> 1;
		g.dxldy = bfe_s(int(w[3] >> 2), 28) >> 1;
		g.dxhdy = bfe_s(int(w[5] >> 2), 28) >> 1;
		g.dxmdy = bfe_s(int(w[7] >> 2), 28) >> 1;
		const uint32_t *p = w + 8;
		if (op & 4)
		{
			// rdp_device.cpp:315-336
			for (int c = 0; c < 4; c++)
			{
				int k = c >> 1;
				bool lo = c & 1;
				a.rgba[c] = int(lo ? merge_lo(p[0 + k], p[4 + k]) : merge_hi(p[0 + k], p[4 + k]));
				a.drgba_dx[c] = int(lo ? merge_lo(p[2 + k], p[6 + k]) : merge_hi(p[2 + k], p[6 + k]));
				a.drgba_de[c] = int(lo ? merge_lo(p[8 + k], p[12 + k]) : merge_hi(p[8 + k], p[12 + k]));
				a.drgba_dy[c] = int(lo ? merge_lo(p[10 + k], p[14 + k]) : merge_hi(p[10 + k], p[14 + k]));
			}
			p += 16;
		}
		if (op & 2)
		{
			// rdp_device.cpp:296-313
			a.stzw[0] = int(merge_hi(p[0], p[4]));
			a.stzw[1] = int(merge_lo(p[0], p[4]));
			a.stzw[3] = int(merge_hi(p[1], p[5]));
			a.dstzw_dx[0] = int(merge_hi(p[2], p[6]));
			a.dstzw_dx[1] = int(merge_lo(p[2], p[6]));
			a.dstzw_dx[3] = int(merge_hi(p[3], p[7]));
			a.dstzw_de[0] = int(merge_hi(p[8], p[12]));
			a.dstzw_de[1] = int(merge_lo(p[8], p[12]));
			a.dstzw_de[3] = int(merge_hi(p[9], p[13]));
			a.dstzw_dy[0] = int(merge_hi(p[10], p[14]));
			a.dstzw_dy[1] = int(merge_lo(p[10], p[14]));
			a.dstzw_dy[3] = int(merge_hi(p[11], p[15]));
			p += 16;
		}
		if (op & 1)
		{
			a.stzw[2] = int(p[0]);
			a.dstzw_dx[2] = int(p[1]);
			a.dstzw_de[2] = int(p[2]);
			a.dstzw_dy[2] = int(p[3]);
		}
	}
	else
	{
		// Rectangles (rdp_device.cpp:713-821).
		uint32_t xl = (w[0] >> 12) & 0xfff, yl = w[0] & 0xfff, xh = (w[1] >> 12) & 0xfff, yh = w[1] & 0xfff;
		if (sf & (RS_COPY | RS_FILL)) yl |= 3;
		g.xh = int(xh << 13);
		g.xl = int(xl << 13);
		g.xm = int(xl << 13);
		g.ym = int(yl);
		g.yl = int(yl);
		g.yh = int(yh);
		g.dxhdy = g.dxmdy = g.dxldy = 0;
		tflags = TRI_FLIP | TRI_DISABLE_UPSCALING;
		if (op == 0x24 || op == 0x25)
		{
			bool rflip = op == 0x25;
			tile = (w[1] >> 24) & 7;
			int sv = int((w[2] >> 16) & 0xffff), tv = int(w[2] & 0xffff);
			int dsdx = bfe_s(int((w[3] >> 16) & 0xffff), 16), dtdy = bfe_s(int(w[3] & 0xffff), 16);
			tflags = TRI_FLIP | (rflip ? TRI_DISABLE_UPSCALING : 0) | ((quirks & 0xffu) ? TRI_DISABLE_UPSCALING : 0) |
			         ((quirks & 0xff00u) ? TRI_NATIVE_LOD : 0);
			a.stzw[0] = shlw(sv, 16);
			a.stzw[1] = shlw(tv, 16);
			if (!rflip)
			{
				a.dstzw_dx[0] = shlw(dsdx, 11);
				a.dstzw_de[1] = shlw(dtdy, 11);
				a.dstzw_dy[1] = shlw(dtdy, 11);
			}
			else
			{
				a.dstzw_dx[1] = shlw(dtdy, 11);
				a.dstzw_de[0] = shlw(dsdx, 11);
				a.dstzw_dy[0] = shlw(dsdx, 11);
			}
			if (sf & RS_COPY) tflags |= TRI_SKIP_XFRAC;
		}
	}

	// ---- fixup_triangle_setup (rdp_renderer.cpp:1402-1423)
	if (g.ym < (g.yh & ~3)) g.ym = 0x7fff;
	if (sf & RS_INTERLACE_FIELD)
	{
		tflags |= TRI_INTERLACE_FIELD;
		if (sf & RS_INTERLACE_KEEP_ODD) tflags |= TRI_INTERLACE_KEEP_ODD;
	}
	if (sf & (RS_COPY | RS_FILL)) tflags |= TRI_FILL_COPY_RASTER;
	g.flags = tflags;
	g.tile = tile;

	// ---- derived setup (rdp_renderer.cpp:910-948), computed from the attributes before prim depth
	RdpPrimShade sh;
	uint32_t prim_color = sb[SB_PRIM_COLOR + 1], env = sb[SB_ENV_COLOR + 1];
	int prim_lod_frac = sb[SB_PRIM_COLOR] & 0xff;
	int min_level = (sb[SB_PRIM_COLOR] >> 8) & 31;
	uint32_t pd = sb[SB_PRIM_DEPTH + 1];
	{
		int dz;
		if (use_prim_depth) dz = pd & 0xffff;
		else
		{
			int dzdx = a.dstzw_dx[2] >> 16, dzdy = a.dstzw_dy[2] >> 16;
			int dzpix = (dzdx < 0 ? (~dzdx & 0x7fff) : dzdx) + (dzdy < 0 ? (~dzdy & 0x7fff) : dzdy);
			if (dzpix >= 0x8000) dzpix = 0x8000;
			else if (dzpix == 0) dzpix = 1;
			else dzpix = 1 << (find_msb(dzpix) + 1);
			dz = dzpix;
		}
		int v = 0;
		if (dz & 0xff00) v |= 8;
		if (dz & 0xf0f0) v |= 4;
		if (dz & 0xcccc) v |= 2;
		if (dz & 0xaaaa) v |= 1;
		sh.dz = uint16_t(dz);
		sh.dz_compressed = uint8_t(v);
	}
	uint64_t conv = (uint64_t(sb[SB_CONVERT]) << 32) | sb[SB_CONVERT + 1];
	int k[6];
	for (int j = 0; j < 6; j++) k[j] = int((conv >> (45 - 9 * j)) & 0x1ff);
	int key_center[3] = { int((sb[SB_KEY_R + 1] >> 8) & 0xff), int((sb[SB_KEY_GB + 1] >> 24) & 0xff),
	                      int((sb[SB_KEY_GB + 1] >> 8) & 0xff) };
	int key_scale[3] = { int(sb[SB_KEY_R + 1] & 0xff), int((sb[SB_KEY_GB + 1] >> 16) & 0xff),
	                     int(sb[SB_KEY_GB + 1] & 0xff) };
	for (int cy = 0; cy < 2; cy++)
	{
		uint8_t *ma = sh.c_muladd[cy], *ms = sh.c_mulsub[cy], *mu = sh.c_mul[cy], *ad = sh.c_add[cy];
		for (int c = 0; c < 4; c++) ma[c] = ms[c] = mu[c] = ad[c] = 0;
		// rdp_renderer.cpp:754-908
		switch (rgb[cy][0]) { case 5: put_rgb(ma, env); break; case 3: put_rgb(ma, prim_color); break; default: break; }
		switch (rgb[cy][1])
		{
		case 5: put_rgb(ms, env); break;
		case 3: put_rgb(ms, prim_color); break;
		case 7: put_rgb(ms, uint32_t(k[4]) << 8); break;
		case 6: ms[0] = uint8_t(key_center[0]); ms[1] = uint8_t(key_center[1]); ms[2] = uint8_t(key_center[2]); break;
		default: break;
		}
		switch (rgb[cy][2])
		{
		case 3: put_rgb(mu, prim_color); break;
		case 5: put_rgb(mu, env); break;
		case 10: put_rgb(mu, 0x01010101u * (prim_color & 0xff)); break;
		case 12: put_rgb(mu, 0x01010101u * (env & 0xff)); break;
		case 14: put_rgb(mu, 0x01010101u * uint32_t(prim_lod_frac)); break;
		case 15: put_rgb(mu, uint32_t(k[5]) << 8); break;
		case 6: mu[0] = uint8_t(key_scale[0]); mu[1] = uint8_t(key_scale[1]); mu[2] = uint8_t(key_scale[2]); break;
		default: break;
		}
		switch (rgb[cy][3]) { case 3: put_rgb(ad, prim_color); break; case 5: put_rgb(ad, env); break; default: break; }
		switch (alp[cy][0]) { case 3: ma[3] = uint8_t(prim_color); break; case 5: ma[3] = uint8_t(env); break; default: break; }
		switch (alp[cy][1]) { case 3: ms[3] = uint8_t(prim_color); break; case 5: ms[3] = uint8_t(env); break; default: break; }
		switch (alp[cy][2])
		{
		case 3: mu[3] = uint8_t(prim_color); break;
		case 5: mu[3] = uint8_t(env); break;
		case 6: mu[3] = uint8_t(prim_lod_frac); break;
		default: break;
		}
		switch (alp[cy][3]) { case 3: ad[3] = uint8_t(prim_color); break; case 5: ad[3] = uint8_t(env); break; default: break; }
	}
	uint32_t fog = sb[SB_FOG_COLOR + 1], blendc = sb[SB_BLEND_COLOR + 1];
	for (int c = 0; c < 4; c++)
	{
		sh.fog[c] = uint8_t(fog >> (24 - 8 * c));
		sh.blend_color[c] = uint8_t(blendc >> (24 - 8 * c));
	}
	sh.fill_color = sb[SB_FILL_COLOR + 1];
	sh.min_lod = uint8_t(min_level);
	for (int j = 0; j < 4; j++) sh.factors[j] = int16_t(2 * bfe_s(k[j], 9) + 1);

	if (use_prim_depth)
	{
		a.stzw[2] = int((pd >> 16) & 0x7fff) << 16;
		a.dstzw_dx[2] = a.dstzw_de[2] = a.dstzw_dy[2] = 0;
	}

	// ---- deduce_static_texture_state / deduce_noise_state / normalize_static_state
	// (rdp_renderer.cpp:1136-1400)
	if (!(sf & (RS_FILL | RS_COPY)))
	{
		bool multi = (sf & RS_MULTI_CYCLE) != 0;
		bool t0 = multi ? (acc_t0(rgb[0], alp[0]) || acc_t1(rgb[1], alp[1])) : acc_t0(rgb[1], alp[1]);
		bool t1 = multi ? (acc_t1(rgb[0], alp[0]) || acc_t0(rgb[1], alp[1])) : false;
		bool pt1 = !multi ? acc_t1(rgb[1], alp[1]) : false;
		bool lodf = multi ? (rgb[0][2] == 13 || alp[0][2] == 0 || rgb[1][2] == 13 || alp[1][2] == 0) : false;
		if (t1 && (sf & RS_CONVERT_ONE)) t0 = true;
		if (t0) sf |= RS_USES_TEXEL0;
		if (t1) sf |= RS_USES_TEXEL1;
		if (pt1) sf |= RS_USES_PIPELINED_TEXEL1;
		if (lodf || (sf & RS_TEX_LOD)) sf |= RS_USES_LOD;
	}
	if ((dither & 3) == 2 || ((dither >> 2) & 3) == 2)
		sf |= RS_NEED_NOISE;
	else if (!(sf & (RS_COPY | RS_FILL)))
	{
		if ((sf & RS_MULTI_CYCLE) && rgb[0][0] == 7) sf |= RS_NEED_NOISE;
		if (rgb[1][0] == 7) sf |= RS_NEED_NOISE;
		if ((sf & RS_MULTI_CYCLE) && rgb[0][0] == 7 && rgb[1][0] == 7) sf |= RS_NEED_NOISE_DUAL;
		if ((sf & (RS_ALPHA_TEST | RS_ALPHA_TEST_DITHER)) == (RS_ALPHA_TEST | RS_ALPHA_TEST_DITHER)) sf |= RS_NEED_NOISE;
	}
	if (sf & RS_FILL)
	{
		sf = RS_FILL;
		dither = 0;
		for (int cy = 0; cy < 2; cy++)
			for (int j = 0; j < 4; j++) rgb[cy][j] = alp[cy][j] = 0;
	}
	else if (sf & RS_COPY)
	{
		// USES_TEXEL0 is kept from previous draws in the reference; copy mode never reads it.
		sf &= (RS_COPY | RS_TLUT | RS_TLUT_TYPE | RS_TEX_LOD | RS_DETAIL | RS_PERSPECTIVE | RS_ALPHA_TEST);
		dither = 0;
		for (int cy = 0; cy < 2; cy++)
			for (int j = 0; j < 4; j++) rgb[cy][j] = alp[cy][j] = 0;
	}
	else
	{
		if ((sf & (RS_MULTI_CYCLE | RS_USES_PIPELINED_TEXEL1)) == 0) sf &= ~(RS_BILERP1 | RS_CONVERT_ONE);
		for (int cy = 0; cy < 2; cy++)
		{
			rgb[cy][0] = norm_muladd(rgb[cy][0]);
			rgb[cy][1] = norm_mulsub(rgb[cy][1]);
			rgb[cy][2] = norm_mul(rgb[cy][2]);
			rgb[cy][3] = norm_add(rgb[cy][3]);
			alp[cy][0] = norm_aaddsub(alp[cy][0]);
			alp[cy][1] = norm_aaddsub(alp[cy][1]);
			alp[cy][2] = norm_amul(alp[cy][2]);
			alp[cy][3] = norm_aaddsub(alp[cy][3]);
		}
	}
	sh.static_flags = sf;
	sh.dither = dither;
	for (int cy = 0; cy < 2; cy++)
		for (int j = 0; j < 4; j++)
		{
			sh.comb_rgb[cy][j] = uint8_t(rgb[cy][j]);
			sh.comb_alpha[cy][j] = uint8_t(alp[cy][j]);
		}
	sh.db_flags = df;
	sh.blend[0][0] = (om1 >> 30) & 3; sh.blend[1][0] = (om1 >> 28) & 3;
	sh.blend[0][1] = (om1 >> 26) & 3; sh.blend[1][1] = (om1 >> 24) & 3;
	sh.blend[0][2] = (om1 >> 22) & 3; sh.blend[1][2] = (om1 >> 20) & 3;
	sh.blend[0][3] = (om1 >> 18) & 3; sh.blend[1][3] = (om1 >> 16) & 3;
	sh.coverage_mode = (om1 >> 8) & 3;
	sh.z_mode = (om1 >> 10) & 3;
	sh.tmem_index = pi.tmem_index;
	sh.tileset = pass.ts_base + pi.tileset;
	sh.prim_index = pass.base_prim_index + pi.seq;
	sh.pass = pass_index;
	sh.pad[0] = sh.pad[1] = sh.pad[2] = 0;

	// ---- span job range (rdp_renderer.cpp:1523-1554)
	int min_sub = max(g.yh, g.scissor[1]);
	int max_sub = min(g.yl - 1, g.scissor[3] - 1);
	int ylo = min_sub >> 2, yhi = max_sub >> 2;
	if (yhi < ylo) { ylo = 0; yhi = -1; }
	g.span_ylo = ylo;
	g.span_yhi = yhi;

	// ---- conservative tile bounding box (rdp_renderer.cpp:994-1060), in the pass's pixels: for an
	// upscaled pass the edges are evaluated at scaled sub-scanlines over every scaled row the
	// primitive's lines cover (the binning test reaches S * yl - 1), with one scaled pixel of
	// margin for the rounding of the scaled edge positions.
	const int sl = int(pass.scale & 3u);
	g.bbox[0] = 1; g.bbox[1] = 0; g.bbox[2] = 0; g.bbox[3] = 0;
	if (g.yl > g.yh && yhi >= ylo)
	{
		int start_y = g.yh & ~3;
		int end_y = (g.yl - 1) | 3;
		start_y = max(g.scissor[1], start_y);
		end_y = min(g.scissor[3] - 1, end_y);
		if (end_y >= start_y)
		{
			bool flip = (tflags & TRI_FLIP) != 0;
			const int sy0 = start_y << sl, sy1 = ((end_y + 1) << sl) - 1, ym = g.ym << sl;
			long long l0, r0, l1, r1, l2, r2, l3, r3;
			interp_x64(g, sy0, flip, l0, r0, sl);
			interp_x64(g, sy1, flip, l1, r1, sl);
			l2 = l3 = l0; r2 = r3 = r0;
			if (ym > sy0 && ym < sy1)
			{
				interp_x64(g, ym, flip, l2, r2, sl);
				interp_x64(g, ym - 1, flip, l3, r3, sl);
			}
			long long sx = min(min(l0, l1), min(l2, l3));
			long long ex = max(max(r0, r1), max(r2, r3));
			long long mr = max(sx < 0 ? -sx : sx, ex < 0 ? -ex : ex);
			if (mr > (2047ll << sl)) { sx = 0; ex = 0x7fffffff; }
			else if (sl) { sx -= 1; ex += 1; }
			sx = max(sx, (long long)((g.scissor[0] >> 2) << sl));
			ex = min(ex, (long long)(((g.scissor[2] + 4) >> 2) << sl));
			ex = min(ex, (long long)pass.fb_width - 1);
			int ty0 = sy0 / 32, ty1 = min(sy1 / 32, int(pass.tiles_y) - 1);
			if (ex >= sx && ty1 >= ty0)
			{
				g.bbox[0] = uint16_t(sx / 8);
				g.bbox[1] = uint16_t(ty0);
				g.bbox[2] = uint16_t(min(int(ex / 8), int(pass.tiles_x) - 1));
				g.bbox[3] = uint16_t(ty1);
			}
		}
	}
	g.pad[0] = 0;
	geom_out[i] = g;
	attr_out[i] = a;
	shade_out[i] = sh;
	if (featbits) featbits[i] = rdp_feature_bits(sh.static_flags, sh.db_flags);
}

// ============================================================================ k_raster: spans
// One scanline of a primitive (the reference's SpanSetup, span_setup.comp): the attribute half
// (RGBA / STZW at the span's base x) and the coverage half (4 sub-scanline x ranges in 16.3,
// the pixel range they touch, validity).  64 bytes, so a row is two full sectors.
struct __align__(16) SpanRow
{
	int rgba[4];
	int stzw[4];
	uint16_t xl[4], xr[4];
	int base_x;
	int start_x, end_x;
	int valid;
};
static_assert(sizeof(SpanRow) == RDP_SPAN_ROW_BYTES, "span row layout");

// interpolate_snapped (span_setup.comp:80-85): whole pixels step by the full derivative, the
// sub-pixels of an upscaled pixel by the derivative over the factor (sl = log2 of the factor).
__device__ __forceinline__ int interp_snapped(int d, int dy, int sl)
{
	return mulw(dy >> sl, d) + mulw(dy & ((1 << sl) - 1), d >> sl);
}

// Attribute half of span_setup.comp:99-150; y is a scanline of the image scaled by 2^sl.
__device__ void span_attr(const RdpPrimGeom &g, const RdpPrimAttr &a, int y, SpanRow &out, int sl = 0)
{
	bool do_offset = (g.flags & TRI_DO_OFFSET) != 0;
	bool skip_xfrac = (g.flags & TRI_SKIP_XFRAC) != 0;
	int dy = y - ((g.yh >> 2) << sl);
	int xh = shlw(g.xh, sl) + mulw(dy, shlw(g.dxhdy, 2));
	int drd[4] = { 0, 0, 0, 0 }, dsd[4] = { 0, 0, 0, 0 };
	if (do_offset)
	{
		xh += mulw(3 << sl, g.dxhdy);
#pragma unroll
		for (int c = 0; c < 4; c++)
		{
			int deh = a.drgba_de[c] & ~0x1ff, dyh = a.drgba_dy[c] & ~0x1ff;
			drd[c] = deh - (deh >> 2) - dyh + (dyh >> 2);
			deh = a.dstzw_de[c] & ~0x1ff;
			dyh = a.dstzw_dy[c] & ~0x1ff;
			dsd[c] = deh - (deh >> 2) - dyh + (dyh >> 2);
		}
	}
	int xfrac = skip_xfrac ? 0 : ((xh >> 7) & 0xff);
#pragma unroll
	for (int c = 0; c < 4; c++)
	{
		int v = a.rgba[c] + interp_snapped(a.drgba_de[c], dy, sl);
		out.rgba[c] = ((v & ~0x1ff) + drd[c] - interp_snapped((a.drgba_dx[c] >> 8) & ~1, xfrac, sl)) & ~0x3ff;
		v = a.stzw[c] + interp_snapped(a.dstzw_de[c], dy, sl);
		out.stzw[c] = ((v & ~0x1ff) + dsd[c] - interp_snapped((a.dstzw_dx[c] >> 8) & ~1, xfrac, sl)) & ~0x3ff;
	}
	out.base_x = xh >> 15;
}

__device__ __forceinline__ int quantize_x(int x) { return (x >> 12) | ((x & 0xfff) != 0 ? 1 : 0); }

// Coverage half of span_setup.comp:152-225; y is a scanline of the image scaled by 2^sl.
__device__ void span_x(const RdpPrimGeom &g, int y, SpanRow &out, int sl = 0)
{
	bool flip = (g.flags & TRI_FLIP) != 0;
	int yh_base = (g.yh & ~3) << sl;
	int ym_base = g.ym << sl;
	int ylo = max(g.yh, g.scissor[1]) << sl;
	int yhi = min(g.yl, g.scissor[3]) << sl;
	int lo_sc = (g.scissor[0] << 1) << sl, hi_sc = (g.scissor[2] << 1) << sl;
	bool all_over = true, all_under = true, all_invalid = true;
	int mn = 0x7fffffff, mx = -0x7fffffff - 1;
#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		int ys = y * 4 + k;
		bool clip_y = ys < ylo || ys >= yhi;
		int xh = shlw(g.xh, sl) + mulw(ys - yh_base, g.dxhdy);
		int xm = shlw(g.xm, sl) + mulw(ys - yh_base, g.dxmdy);
		int xl = shlw(g.xl, sl) + mulw(ys - ym_base, g.dxldy);
		if (ys < ym_base) xl = xm;
		xl = bfe_s(xl, 27 + sl);
		xh = bfe_s(xh, 27 + sl);
		int hs = quantize_x(xh), ls = quantize_x(xl);
		int l = flip ? hs : ls, r = flip ? ls : hs;
		bool invalid = ((l >> 1) > (r >> 1)) || clip_y;
		all_over = all_over && (min(l, r) >= hi_sc);
		all_under = all_under && (max(l, r) < lo_sc);
		l = min(max(l, lo_sc), hi_sc);
		r = min(max(r, lo_sc), hi_sc);
		if (invalid) { l = 0xffff; r = 0; }
		all_invalid = all_invalid && invalid;
		out.xl[k] = uint16_t(l);
		out.xr[k] = uint16_t(r);
		mn = min(mn, l);
		mx = max(mx, r);
	}
	out.start_x = mn >> 3;
	out.end_x = mx >> 3;
	bool valid = !all_invalid && !all_over && !all_under;
	if ((g.flags & TRI_INTERLACE_FIELD) && (((y >> sl) & 1) != int((g.flags & TRI_INTERLACE_KEEP_ODD) != 0))) valid = false;
	out.valid = valid ? 1 : 0;
}

// ============================================================================ k_bin
// binning.h:58-144; lo/hi are pixels of the image scaled by 2^sl.
__device__ bool bin_primitive(const RdpPrimGeom &g, int lox, int loy, int hix, int hiy, int sl = 0)
{
	loy = max(loy, (g.scissor[1] >> 2) << sl);
	hiy = min(hiy, (((g.scissor[3] + 3) >> 2) << sl) - 1);
	int start_y = max(loy * 4, g.yh << sl);
	int end_y = min(hiy * 4 + 3, (g.yl << sl) - 1);
	if (end_y < start_y) return false;
	bool flip = (g.flags & TRI_FLIP) != 0;
	const int ym = g.ym << sl;
	int ys[4] = { start_y, end_y, clampi(ym - 1, start_y, end_y), clampi(ym, start_y, end_y) };
	const long long yh_base = (long long)((g.yh & ~3) << sl), ym_base = ym;
	int xmin = 0x7fffffff, xmax = -0x7fffffff - 1, mr = 0;
#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		long long xh = (long long)shlw(g.xh, sl) + (long long)(ys[k] - yh_base) * g.dxhdy;
		long long xm = (long long)shlw(g.xm, sl) + (long long)(ys[k] - yh_base) * g.dxmdy;
		long long xl = (long long)shlw(g.xl, sl) + (long long)(ys[k] - ym_base) * g.dxldy;
		if (ys[k] < ym) xl = xm;
		xh = min(max(xh, -2147483648LL), 2147483647LL);
		xl = min(max(xl, -2147483648LL), 2147483647LL);
		int hs = int(xh) >> 15, ls = int(xl) >> 15;
		int l = flip ? hs : ls, r = flip ? ls : hs;
		xmin = min(xmin, l);
		xmax = max(xmax, r);
		mr = max(mr, max(abs(l), abs(r)));
	}
	int rx0, rx1;
	if (mr <= (2047 << sl)) { rx0 = xmin; rx1 = xmax; }
	else { rx0 = 0; rx1 = 0x7fffffff; }
	int x_bias = (g.flags & TRI_FILL_COPY_RASTER) ? 4 : 3;
	int sx0 = (g.scissor[0] >> 2) << sl, sx1 = (((g.scissor[2] + x_bias) >> 2) << sl) - 1;
	rx0 = clampi(rx0, sx0, sx1);
	rx1 = clampi(rx1, sx0, sx1);
	rx0 = max(rx0, lox);
	rx1 = min(rx1, hix);
	return rx0 <= rx1;
}

// A warp takes 32 consecutive primitives and tests their (primitive, tile) pairs flattened: the
// exclusive prefix of the primitives' tile-box sizes numbers the warp's tests, lane l takes tests
// l, l + 32, ... and finds its primitive by binary search of the prefix, so the lanes stay busy
// whatever the mix of box sizes.  With `prim_pairs`, also writes each primitive's number of binned
// tiles (its pairs), counted in shared memory.  Without it the grid's y dimension may split a
// warp's tests over several warps (launches of a few large primitives, such as a frame's clears):
// warp k takes tests k*32 + lane, then every 32*gridDim.y-th further.
__global__ void __launch_bounds__(256) k_bin(uint32_t num_prims, const RdpPrimGeom *__restrict__ geom,
                                            const RdpPrimShade *__restrict__ shade, const RdpPass *__restrict__ passes,
                                            uint32_t *__restrict__ tile_counts, uint32_t *__restrict__ prim_pairs)
{
	__shared__ uint32_t s_binned[8][32];
	const uint32_t prim = blockIdx.x * blockDim.x + threadIdx.x;
	const int lane = int(threadIdx.x & 31), wib = int(threadIdx.x >> 5);
	const uint32_t warp_first = prim - uint32_t(lane);
	if (warp_first >= num_prims) return; // the whole warp
	uint32_t count = 0;
	if (prim < num_prims)
	{
		const RdpPrimGeom &g = geom[prim];
		if (g.bbox[2] >= g.bbox[0] && g.bbox[3] >= g.bbox[1])
			count = uint32_t(g.bbox[2] - g.bbox[0] + 1) * uint32_t(g.bbox[3] - g.bbox[1] + 1);
	}
	uint32_t incl = count;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
		const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
		if (lane >= o) incl += y;
	}
	const uint32_t first = incl - count, total = __shfl_sync(0xffffffffu, incl, 31);
	if (prim_pairs) s_binned[wib][lane] = 0u;
	__syncwarp();
	for (uint32_t f0 = blockIdx.y * 32u; f0 < total; f0 += 32u * gridDim.y)
	{
		const uint32_t f = f0 + uint32_t(lane);
		// The primitive holding test f: the largest j with first_j <= f (first_0 = 0).
		int j = 0;
		uint32_t fj = 0;
#pragma unroll
		for (int step = 16; step > 0; step >>= 1)
		{
			const uint32_t c = __shfl_sync(0xffffffffu, first, j + step);
			if (c <= f)
			{
				j += step;
				fj = c;
			}
		}
		if (f >= total) continue;
		const uint32_t p = warp_first + uint32_t(j);
		const RdpPrimGeom &g = geom[p];
		const RdpPass &pass = passes[shade[p].pass];
		const int t = int(f - fj);
		const int tw = g.bbox[2] - g.bbox[0] + 1;
		const int tx = g.bbox[0] + t % tw, ty = g.bbox[1] + t / tw;
		const int lox = tx * 8, loy = ty * 8;
		const int hix = min(lox + 7, int(pass.fb_width) - 1), hiy = min(loy + 7, int(pass.fb_height) - 1);
		if (bin_primitive(g, lox, loy, hix, hiy, int(pass.scale & 3u)))
		{
			const uint32_t local = p - pass.prim_begin;
			const uint32_t tl = uint32_t(ty) * pass.tiles_x + uint32_t(tx);
			atomicOr(&pass.masks[size_t(tl) * pass.mask_words + (local >> 5)], 1u << (local & 31));
			// Upscaled and fill-only launches render from the bitmasks alone (no pair list).
			if (tile_counts) atomicAdd(&tile_counts[pass.tile_item_begin + tl], 1u);
			if (prim_pairs) atomicAdd(&s_binned[wib][j], 1u);
		}
	}
	if (prim_pairs)
	{
		__syncwarp();
		if (prim < num_prims) prim_pairs[prim] = s_binned[wib][lane];
	}
}

// ============================================================================ k_span
// Spans of the scanlines of every primitive that can have tiles (span_setup.comp), computed once
// per primitive row for all the primitive's tiles: rows span_ylo .. the last shaded row + 1 (the
// pipelined texel1 peek reads the next row).  A CTA takes `chunk` (<= SPAN_THREADS) consecutive
// primitives: one thread per primitive counts its rows, a CTA scan gives each primitive its first
// row, one atomic on the launch's 64-bit row counter (k_scan resets it) places the CTA's rows,
// and then one thread per row computes it (the row's primitive found by binary search of the
// scan).  The host sizes `chunk` to the launch, so that a few tall primitives (a clear) still
// spread over many CTAs while large launches take few atomics.  A CTA whose rows would not fit
// `capacity` writes none; the launch then takes k_raster (write_ctrl flags it) and the host
// grows the buffer to the count seen.
constexpr int SPAN_THREADS = 256;

__global__ void __launch_bounds__(SPAN_THREADS, 6) k_span(uint32_t num_prims, const RdpPrimGeom *__restrict__ geom,
                                                      const RdpPrimAttr *__restrict__ attr,
                                                      const RdpPrimShade *__restrict__ shade,
                                                      const RdpPass *__restrict__ passes, SpanRow *__restrict__ spans,
                                                      uint32_t capacity, uint32_t *__restrict__ prim_rows,
                                                      unsigned long long *__restrict__ row_counter, uint32_t chunk)
{
	constexpr int NW = SPAN_THREADS / 32;
	__shared__ uint32_t s_first[SPAN_THREADS + 1]; // first row of each primitive in the CTA, then the total
	__shared__ uint32_t s_warp[NW];
	__shared__ unsigned long long s_base;
	const uint32_t t = threadIdx.x, lane = t & 31, wid = t >> 5;
	const uint32_t p0 = blockIdx.x * chunk, prim = p0 + t;
	uint32_t nrows = 0;
	if (t < chunk && prim < num_prims)
	{
		const RdpPrimGeom &g = geom[prim];
		const int r_last = min(g.span_yhi, int(passes[shade[prim].pass].fb_height) - 1);
		const bool has_tiles = g.bbox[2] >= g.bbox[0] && g.bbox[3] >= g.bbox[1];
		if (has_tiles && r_last >= g.span_ylo) nrows = uint32_t(r_last - g.span_ylo + 2);
	}
	uint32_t x = nrows;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
		const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= uint32_t(o)) x += y;
	}
	if (lane == 31) s_warp[wid] = x;
	__syncthreads();
	if (wid == 0)
	{
		uint32_t w = lane < uint32_t(NW) ? s_warp[lane] : 0u;
#pragma unroll
		for (int o = 1; o < NW; o <<= 1)
		{
			const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
			if (lane >= uint32_t(o)) w += y;
		}
		if (lane < uint32_t(NW)) s_warp[lane] = w;
	}
	__syncthreads();
	const uint32_t first = (wid ? s_warp[wid - 1] : 0u) + x - nrows, total = s_warp[NW - 1];
	s_first[t] = first;
	if (t == 0)
	{
		s_first[SPAN_THREADS] = total;
		s_base = total ? atomicAdd(row_counter, (unsigned long long)total) : 0ull;
	}
	__syncthreads();
	const unsigned long long base = s_base;
	if (t < chunk && prim < num_prims) prim_rows[prim] = uint32_t(base + first);
	if (base + total > capacity) return;
	for (uint32_t i = t; i < total; i += SPAN_THREADS)
	{
		// The largest k with s_first[k] <= i: the primitive whose rows hold row i.
		uint32_t lo = 0, hi = chunk;
		while (hi - lo > 1)
		{
			const uint32_t mid = (lo + hi) >> 1;
			if (s_first[mid] <= i) lo = mid;
			else hi = mid;
		}
		const uint32_t pk = p0 + lo;
		const RdpPrimGeom &g = geom[pk];
		const int y = g.span_ylo + int(i - s_first[lo]);
		SpanRow row;
		span_x(g, y, row);
		span_attr(g, attr[pk], y, row);
		spans[base + i] = row;
	}
}

// ============================================================================ k_tmem
__device__ __forceinline__ uint8_t rd8(const RdpPass &p, uint32_t a) { return p.rdram[a & (p.rdram_size - 1)]; }
__device__ __forceinline__ uint16_t rd16(const RdpPass &p, uint32_t i)
{
	uint32_t b = (i * 2) & (p.rdram_size - 1);
	return *reinterpret_cast<const uint16_t *>(p.rdram + b);
}
__device__ __forceinline__ uint32_t rd32(const RdpPass &p, uint32_t i)
{
	uint32_t b = (i * 4) & (p.rdram_size - 1);
	return *reinterpret_cast<const uint32_t *>(p.rdram + b);
}

__device__ __forceinline__ int upload_t(int offset, float inv_stride)
{
	return int(__fmul_rn(__fadd_rn(float(offset), 0.5f), inv_stride));
}

// tmem_update.comp:108-317
__device__ bool tmem_32(const RdpPass &ps, const RdpUpload &info, int tmem16_index, bool upper, bool yuv, uint32_t &value)
{
	int tmem16_offset = (info.tmem_offset & 0x7ff) >> 1;
	int stride = info.tmem_stride_words;
	int pixel_offset = (tmem16_index - tmem16_offset) & 0x3ff;
	int ux, uy, uxx = 0;
	if (info.mode == 2)
	{
		int wo = pixel_offset >> 1;
		if (stride == 0)
		{
			int f = wo & ~1, s = f + 1;
			int ft = mulw(f, info.dxt) >> 16, st = mulw(s, info.dxt) >> 16;
			if (ft != st)
			{
				int fw = f ^ (ft & 1), sw = s ^ (st & 1);
				if (sw == wo) uxx = (st & 1) << 1;
				else if (fw == wo) uxx = (ft & 1) << 1;
				else return false;
			}
			else
				uxx ^= (ft & 1) << 1;
		}
		else
		{
			int min_t = upload_t(wo & ~1, info.min_t_mod);
			int max_t = upload_t(wo | 1, info.max_t_mod);
			int max_wc = (wo | 1) - stride * min_t;
			int min_wc = (wo & ~1) - stride * max_t;
			min_t = max(min_t, mulw(min_wc, info.dxt) >> 16);
			max_t = min(max_t, mulw(max_wc, info.dxt) >> 16);
			bool found = false;
			for (int t = max_t; t >= min_t; t--)
			{
				int c1 = (wo & ~1) - stride * t, c2 = (wo | 1) - stride * t;
				int t1 = mulw(c1, info.dxt) >> 16, t2 = mulw(c2, info.dxt) >> 16;
				if (((c2 + t2 * stride) ^ (t2 & 1)) == wo)
				{
					found = true;
					pixel_offset = (c2 << 1) + (pixel_offset & 1);
					break;
				}
				else if (((c1 + t1 * stride) ^ (t1 & 1)) == wo)
				{
					found = true;
					pixel_offset = (c1 << 1) + (pixel_offset & 1);
					break;
				}
			}
			if (!found) return false;
		}
		ux = pixel_offset;
		uy = 0;
	}
	else if (stride == 0)
	{
		ux = pixel_offset;
		uy = info.height - 1;
	}
	else
	{
		uy = upload_t(pixel_offset, info.inv_tmem_stride_words);
		ux = pixel_offset - uy * stride;
		if (uy >= info.height)
		{
			ux += stride * (uy - info.height + 1);
			uy = info.height - 1;
		}
	}
	int last_x = ux ^ ((uy & 1) << 1);
	if (last_x >= info.width && uy > 0)
	{
		uy--;
		ux += stride;
	}
	int it = 0;
	ux ^= ((uy & 1) << 1) | uxx;
	if (info.vram_size == 3 || yuv) it = 4 * (ux & ~1);
	else if (info.vram_size == 2)
	{
		if (ux & 2)
		{
			if (uy > 0)
			{
				uy--;
				ux += stride;
				ux ^= 2;
			}
			else
				return false;
		}
		it = 2 * (ux & ~1);
	}
	else if (info.vram_size == 1)
	{
		for (int k = 0; k < 4 && uy > 0 && (ux & 6) != 0; k++)
		{
			uy--;
			ux += stride;
			ux ^= 2;
		}
		if (ux & 6) return false;
		it = ux & ~1;
	}
	if (ux >= info.width) return false;
	int line = info.vram_addr + shlw(mulw(uy, info.vram_width), info.vram_size - 1);
	int addr = line + it + 4 * (ux & 1);
	uint32_t word;
	if ((addr & 3) == 0) word = rd32(ps, uint32_t(addr) >> 2);
	else
		word = (uint32_t(rd8(ps, uint32_t(addr) ^ 3)) << 24) | (uint32_t(rd8(ps, uint32_t(addr + 1) ^ 3)) << 16) |
		       (uint32_t(rd8(ps, uint32_t(addr + 2) ^ 3)) << 8) | uint32_t(rd8(ps, uint32_t(addr + 3) ^ 3));
	if (yuv)
	{
		if (upper) word = (((word >> 16) & 0xffu) << 8) | (word & 0xffu);
		else word = (((word >> 24) & 0xffu) << 8) | ((word >> 8) & 0xffu);
	}
	else
	{
		word >>= 16u - 16u * uint32_t(upper);
		word &= 0xffffu;
	}
	value = word;
	return true;
}

// tmem_update.comp:319-459
__device__ bool tmem_16(const RdpPass &ps, const RdpUpload &info, int tmem16_index, uint32_t &value)
{
	int tmem16_offset = (info.tmem_offset & 0xfff) >> 1;
	int stride = info.tmem_stride_words;
	int pixel_offset = (tmem16_index - tmem16_offset) & 0x7ff;
	int ux, uy, uxx = 0;
	if (info.mode == 2)
	{
		int wo = pixel_offset >> 2;
		if (stride == 0)
			uxx = ((mulw(wo, info.dxt) >> 16) & 1) << 1;
		else
		{
			int min_t = upload_t(wo, info.min_t_mod);
			int max_t = upload_t(wo, info.max_t_mod);
			int max_wc = wo - stride * min_t;
			int min_wc = wo - stride * max_t;
			min_t = max(min_t, mulw(min_wc, info.dxt) >> 16);
			max_t = min(max_t, mulw(max_wc, info.dxt) >> 16);
			bool found = false;
			for (int t = max_t; t >= min_t; t--)
			{
				int cand = wo - stride * t;
				int ct = mulw(cand, info.dxt) >> 16;
				if (cand + ct * stride == wo)
				{
					found = true;
					uxx = (ct & 1) << 1;
					pixel_offset = (cand << 2) + (pixel_offset & 3);
				}
			}
			if (!found) return false;
		}
		ux = pixel_offset;
		uy = 0;
	}
	else if (stride == 0)
	{
		ux = pixel_offset;
		uy = info.height - 1;
	}
	else
	{
		uy = upload_t(pixel_offset, info.inv_tmem_stride_words);
		ux = pixel_offset - uy * stride;
		if (uy >= info.height)
		{
			ux += stride * (uy - info.height + 1);
			uy = info.height - 1;
		}
	}
	int it = 0;
	if (info.tmem_size != info.vram_size)
	{
		if (info.vram_size - info.tmem_size == 1)
		{
			it = (ux & ~3) * 4;
			if ((ux & ~3) + 2 < (info.vram_effective_width >> (3 - info.vram_size))) it += 8;
		}
		else if (info.tmem_size == 2 && info.vram_size == 1)
		{
			if (ux & 4)
			{
				if ((stride & 4) != 0 && uy > 0)
				{
					uy--;
					ux += stride;
				}
				else
					return false;
			}
			it = ux & ~3;
		}
	}
	else
		it = (ux & ~3) * 2;
	if (ux >= info.width) return false;
	int line = info.vram_addr + shlw(mulw(uy, info.vram_width), info.vram_size - 1);
	ux ^= ((uy & 1) << 1) | uxx;
	int addr = line + it + 2 * (ux & 3);
	uint32_t word;
	if ((addr & 1) == 0) word = rd16(ps, (uint32_t(addr) >> 1) ^ 1u);
	else word = (uint32_t(rd8(ps, uint32_t(addr) ^ 3)) << 8) | uint32_t(rd8(ps, uint32_t(addr + 1) ^ 3));
	value = word;
	return true;
}

// tmem_update.comp:461-544
__device__ bool tmem_lut(const RdpPass &ps, const RdpUpload &info, int tmem16_index, uint32_t &value)
{
	int tmem16_offset = (info.tmem_offset & 0xfff) >> 1;
	int po = (tmem16_index - tmem16_offset) & 0x7ff;
	int splat;
	int d = info.vram_size - info.tmem_size;
	if (d == 2)
	{
		splat = (po >> 2) << (info.vram_size - 2);
		if (splat >= info.vram_effective_width) return false;
	}
	else if (d == 1)
	{
		if (po & 4) return false;
		int shamt = info.tmem_size + (info.vram_size == 2 ? 2 : 0);
		splat = (po & ~7) >> shamt;
		if (splat >= info.vram_effective_width) return false;
	}
	else if (d == 0)
	{
		if (po & 0xc) return false;
		int shamt = info.tmem_size + (info.vram_size == 2 ? 2 : 0);
		splat = (po & ~3) >> shamt;
		if (splat >= info.vram_effective_width) return false;
	}
	else if (d == -1)
	{
		if (po & 0x1c) return false;
		splat = (po >> info.tmem_size) & ~7;
		if (splat >= info.vram_effective_width) return false;
	}
	else
	{
		int sp = ((po >> 2) * 2) * 2;
		if (sp + 2 < info.vram_effective_width) sp += 2;
		if (sp >= info.vram_effective_width) return false;
		splat = sp;
	}
	int addr = info.vram_addr + shlw(splat, info.vram_size - 1);
	addr += 2 * (addr & 1) * (po & 3);
	uint32_t word;
	if ((addr & 1) == 0) word = rd16(ps, (uint32_t(addr) >> 1) ^ 1u);
	else word = (uint32_t(rd8(ps, uint32_t(addr) ^ 3)) << 8) | uint32_t(rd8(ps, uint32_t(addr + 1) ^ 3));
	value = word;
	return true;
}

// Phase 1: every (upload, TMEM word) pair independently -- does upload u write word w, and with
// what value?  Written values land in snapshot u+1; unwritten words are marked in a bitmask.  One
// CTA per upload of the launch (the launch's uploads are the TMEM passes' uploads, concatenated in
// pass order); the CTA finds its pass by binary search over their first uploads.
__global__ void __launch_bounds__(256, 8) k_tmem_apply(const RdpPass *__restrict__ passes, const uint32_t *__restrict__ pass_list,
                             uint32_t num_tmem_passes, const RdpUpload *__restrict__ uploads,
                             uint32_t *__restrict__ keep_bits)
{
	const uint32_t g = blockIdx.x;
	uint32_t lo = 0, hi = num_tmem_passes;
	while (hi - lo > 1)
	{
		const uint32_t mid = (lo + hi) >> 1;
		if (passes[pass_list[mid]].upload_begin <= g) lo = mid;
		else hi = mid;
	}
	const RdpPass &ps = passes[pass_list[lo]];
	const uint32_t u = g - ps.upload_begin;
	if (g < ps.upload_begin || u >= ps.upload_count) return;
	RdpUpload info = uploads[g];
	uint16_t *dst = ps.tmem_snapshots + size_t(u + 1) * 2048;
	uint32_t *keep = keep_bits + size_t(g) * 64;
	for (int gid = threadIdx.x; gid < 2048; gid += blockDim.x)
	{
		int idx = gid ^ 1;
		bool upper = idx >= 0x400;
		uint32_t v = 0;
		bool wrote;
		if (info.mode == 1) wrote = tmem_lut(ps, info, idx, v);
		else
		{
			bool yuv = info.tmem_fmt == 1;
			if (info.tmem_size == 3 || yuv) wrote = tmem_32(ps, info, idx & 0x3ff, upper, yuv, v);
			else wrote = tmem_16(ps, info, idx, v);
		}
		if (wrote) dst[gid] = uint16_t(v);
		unsigned m = __ballot_sync(0xffffffffu, !wrote);
		if ((threadIdx.x & 31) == 0) keep[gid >> 5] = m;
	}
}

// Phase 2: carry the previous snapshot's value through uploads that did not write a word
// (tmem_update.comp:546-576: instance i+1 = instance i with upload i applied).  One CTA per
// (pass, 32 TMEM words), lane = word; its TMEM_CARRY_WARPS warps split the uploads into chunks:
// each warp finds the last value its chunk writes, the chunks' carry-ins are chained in shared
// memory, then every warp fills its chunk.  A warp reads each upload's keep word of its 32 words
// (one broadcast load) and tests its lane's bit; TMEM_CARRY_AHEAD uploads' keep words and written
// snapshot values are loaded together ahead of the stores that carry them on.
constexpr int TMEM_CARRY_WARPS = 32; // 8: +0.19 ms per batched sync point, 16: +0.05 ms
constexpr int TMEM_CARRY_AHEAD = 8;  // uploads whose loads are issued together

__global__ void __launch_bounds__(TMEM_CARRY_WARPS * 32, 2) k_tmem_carry(const RdpPass *__restrict__ passes,
                                                                       const uint32_t *__restrict__ pass_list,
                                                                       const uint32_t *__restrict__ keep_bits)
{
	__shared__ uint16_t s_last[TMEM_CARRY_WARPS][32];
	__shared__ uint8_t s_has[TMEM_CARRY_WARPS][32];
	__shared__ uint16_t s_in[TMEM_CARRY_WARPS][32];
	const RdpPass &ps = passes[pass_list[blockIdx.y]];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int gid = blockIdx.x * 32 + lane;
	const uint32_t n = ps.upload_count;
	const uint32_t chunk = (n + TMEM_CARRY_WARPS - 1) / TMEM_CARRY_WARPS;
	const uint32_t u0 = min(n, uint32_t(warp) * chunk), u1 = min(n, u0 + chunk);
	// Word gid of snapshot s (the state after s uploads): col[s * 2048].
	uint16_t *col = ps.tmem_snapshots + gid;
	// This CTA's keep word of upload u: keep_words[u * 64] (bit = lane: the upload left the word alone).
	const uint32_t *keep_words = keep_bits + size_t(ps.upload_begin) * 64 + blockIdx.x;

	int last_u = -1;
	for (uint32_t ub = u0; ub < u1; ub += TMEM_CARRY_AHEAD)
	{
		uint32_t kw[TMEM_CARRY_AHEAD];
#pragma unroll
		for (int k = 0; k < TMEM_CARRY_AHEAD; k++)
			kw[k] = ub + uint32_t(k) < u1 ? keep_words[size_t(ub + uint32_t(k)) * 64] : 0xffffffffu;
#pragma unroll
		for (int k = 0; k < TMEM_CARRY_AHEAD; k++)
			if (!((kw[k] >> lane) & 1u)) last_u = int(ub) + k;
	}
	s_last[warp][lane] = last_u >= 0 ? col[size_t(last_u + 1) * 2048] : uint16_t(0);
	s_has[warp][lane] = last_u >= 0;
	__syncthreads();
	if (warp == 0)
	{
		uint16_t v = ps.tmem_state[gid];
		col[0] = v;
		for (int w = 0; w < TMEM_CARRY_WARPS; w++)
		{
			s_in[w][lane] = v;
			if (s_has[w][lane]) v = s_last[w][lane];
		}
		ps.tmem_state[gid] = v;
	}
	__syncthreads();
	uint16_t value = s_in[warp][lane];
	for (uint32_t ub = u0; ub < u1; ub += TMEM_CARRY_AHEAD)
	{
		bool wrote[TMEM_CARRY_AHEAD];
		uint16_t got[TMEM_CARRY_AHEAD];
#pragma unroll
		for (int k = 0; k < TMEM_CARRY_AHEAD; k++)
		{
			const uint32_t u = ub + uint32_t(k);
			wrote[k] = u < u1 && !((keep_words[size_t(u) * 64] >> lane) & 1u);
			got[k] = wrote[k] ? col[size_t(u + 1) * 2048] : uint16_t(0);
		}
#pragma unroll
		for (int k = 0; k < TMEM_CARRY_AHEAD; k++)
		{
			const uint32_t u = ub + uint32_t(k);
			if (u >= u1) break;
			if (wrote[k]) value = got[k];
			else col[size_t(u + 1) * 2048] = value;
		}
	}
}

// ============================================================================ k_raster: per-pixel maths
__device__ __forceinline__ int clamp_9bit(int c) { return clampi(bfe_s(c - 0x80, 9) + 0x80, 0, 0xff); }
__device__ __forceinline__ int special_expand(int v) { return bfe_s(v - 0x80, 9) + 0x80; }

__device__ __forceinline__ int clamp_z(int z)
{
	z -= 1 << 17;
	z = int(unsigned(z) << 13) >> 13;
	z += 1 << 17;
	return clampi(z, 0, 0x3ffff);
}

__device__ __forceinline__ uint32_t reseed_noise(uint32_t x, uint32_t y, uint32_t p)
{
	const uint32_t P = 1103515245u;
	uint32_t s0 = x, s1 = y, s2 = p;
#pragma unroll
	for (int k = 0; k < 3; k++)
	{
		uint32_t n0 = ((s0 >> 8) ^ s1) * P;
		uint32_t n1 = ((s1 >> 8) ^ s2) * P;
		uint32_t n2 = ((s2 >> 8) ^ s0) * P;
		s0 = n0; s1 = n1; s2 = n2;
	}
	return s0 >> 16;
}

__device__ void persp_divide(int s, int t, int w, int &os, int &ot, bool &overflow)
{
	bool w_carry = w <= 0;
	w &= 0x7fff;
	int shift = min(14 - find_msb(w), 14);
	int normout = shlw(w, shift) & 0x3fff;
	int wnorm = normout & 0xff;
	int idx = normout >> 8;
	int rcp = ((-int(g_persp_slope[idx]) * 4 * wnorm) >> 10) + g_persp_base[idx];
	int prod0 = mulw(s, rcp), prod1 = mulw(t, rcp);
	int temp_mask = ((1 << 30) - 1) & -((1 << 29) >> shift);
	int oob0 = prod0 & temp_mask, oob1 = prod1 & temp_mask;
	int t0, t1;
	if (shift != 14)
	{
		t0 = prod0 = prod0 >> (13 - shift);
		t1 = prod1 = prod1 >> (13 - shift);
	}
	else
	{
		t0 = shlw(prod0, 1);
		t1 = shlw(prod1, 1);
	}
	if (oob0 != 0 && oob0 != temp_mask)
	{
		t0 = (prod0 & (1 << 29)) == 0 ? 0x7fff : -0x8000;
		overflow = true;
	}
	if (oob1 != 0 && oob1 != temp_mask)
	{
		t1 = (prod1 & (1 << 29)) == 0 ? 0x7fff : -0x8000;
		overflow = true;
	}
	if (w_carry)
	{
		t0 = t1 = 0x7fff;
		overflow = true;
	}
	os = clampi(t0, -0x10000, 0xffff);
	ot = clampi(t1, -0x10000, 0xffff);
}

__device__ __forceinline__ void st_div(int s, int t, int w, bool persp, int &os, int &ot, bool &ov)
{
	if (persp) persp_divide(s, t, w, os, ot, ov);
	else { os = s; ot = t; }
}

// ---------------------------------------------------------------------------- textures (texture.h)
struct T4 { int v[4]; };

__device__ __forceinline__ uint32_t tm16(const uint16_t *tm, uint32_t i) { return __ldg(tm + (i & 2047)); }
__device__ __forceinline__ uint32_t tm8(const uint16_t *tm, uint32_t i) { return (tm16(tm, i >> 1) >> ((i & 1) * 8)) & 0xff; }

__device__ __forceinline__ T4 cvt_rgba16(uint32_t w)
{
	T4 r;
#pragma unroll
	for (int c = 0; c < 3; c++)
	{
		uint32_t x = (w >> (11 - 5 * c)) & 31u;
		r.v[c] = int((x << 3) | (x >> 2));
	}
	r.v[3] = int((w & 1u) * 0xffu);
	return r;
}
__device__ __forceinline__ T4 cvt_ia16(uint32_t w)
{
	int i = int(w >> 8), al = int(w & 0xff);
	return { { i, i, i, al } };
}
__device__ __forceinline__ T4 splat4(int v) { return { { v, v, v, v } }; }

__device__ __forceinline__ uint32_t byte_idx(const RdpTile &t, int sb, int tv, uint32_t wrap)
{
	uint32_t off = (t.offset + t.stride * uint32_t(tv) + uint32_t(sb)) & wrap;
	return (off ^ ((uint32_t(tv) & 1u) << 2)) ^ 3u;
}
__device__ __forceinline__ uint32_t hw_idx(const RdpTile &t, int s, int tv, uint32_t wrap)
{
	uint32_t off = (t.offset + t.stride * uint32_t(tv) + uint32_t(s) * 2u) & wrap;
	return ((off >> 1) ^ ((uint32_t(tv) & 1u) << 1)) ^ 1u;
}

__device__ __noinline__ T4 fetch_texel(const uint16_t *tm, const RdpTile &t, int s, int tv, bool tlut, bool tlut_type, uint32_t lut_off,
                          uint32_t ax)
{
	if (tlut)
	{
		uint32_t w;
		switch (t.size)
		{
		case 0:
		{
			uint32_t idx = byte_idx(t, s >> 1, tv, 0x7ff);
			uint32_t v = (tm8(tm, idx) >> ((~uint32_t(s) & 1u) * 4)) & 0xf;
			v |= uint32_t(t.palette) << 4;
			w = tm16(tm, 0x400 | (((v << 2) + lut_off) ^ ax));
			break;
		}
		case 1:
		{
			uint32_t v = tm8(tm, byte_idx(t, s, tv, 0x7ff));
			w = tm16(tm, 0x400 | (((v << 2) + lut_off) ^ ax));
			break;
		}
		default:
		{
			uint32_t v = tm16(tm, hw_idx(t, s, tv, 0x7ff));
			w = tm16(tm, 0x400 | ((((v >> 6) & ~3u) + lut_off) ^ ax));
			break;
		}
		}
		return tlut_type ? cvt_ia16(w) : cvt_rgba16(w);
	}
	switch (t.fmt)
	{
	case 0: // RGBA
		switch (t.size)
		{
		case 0:
		{
			uint32_t v = (tm8(tm, byte_idx(t, s >> 1, tv, 0xfff)) >> ((~uint32_t(s) & 1u) * 4)) & 0xf;
			return splat4(int(v | (v << 4)));
		}
		case 1: return splat4(int(tm8(tm, byte_idx(t, s, tv, 0xfff))));
		case 2: return cvt_rgba16(tm16(tm, hw_idx(t, s, tv, 0xfff)));
		default:
		{
			uint32_t idx = hw_idx(t, s, tv, 0x7ff) & 2047;
			uint32_t lo = tm16(tm, idx), hi = tm16(tm, idx | 0x400);
			return { { int(lo >> 8), int(lo & 0xff), int(hi >> 8), int(hi & 0xff) } };
		}
		}
	case 2: // CI
		switch (t.size)
		{
		case 0:
		{
			uint32_t v = (tm8(tm, byte_idx(t, s >> 1, tv, 0xfff)) >> ((~uint32_t(s) & 1u) * 4)) & 0xf;
			return splat4(int(v | (uint32_t(t.palette) << 4)));
		}
		case 1: return splat4(int(tm8(tm, byte_idx(t, s, tv, 0xfff))));
		default:
		{
			uint32_t v = tm16(tm, hw_idx(t, s, tv, 0xfff));
			int x = int(v >> 8), y = int(v & 0xff);
			return { { x, y, x, y } };
		}
		}
	case 3: // IA
		switch (t.size)
		{
		case 0:
		{
			uint32_t v = (tm8(tm, byte_idx(t, s >> 1, tv, 0xfff)) >> ((~uint32_t(s) & 1u) * 4)) & 0xf;
			uint32_t i = v & 0xe;
			i = (i << 4) | (i << 1) | (i >> 2);
			return { { int(i), int(i), int(i), int((v & 1) * 0xff) } };
		}
		case 1:
		{
			uint32_t v = tm8(tm, byte_idx(t, s, tv, 0xfff));
			uint32_t i = v >> 4, al = v & 0xf;
			al |= al << 4;
			i |= i << 4;
			return { { int(i), int(i), int(i), int(al) } };
		}
		case 2: return cvt_ia16(tm16(tm, hw_idx(t, s, tv, 0xfff)));
		default:
		{
			uint32_t v = tm16(tm, hw_idx(t, s, tv, 0xfff));
			int x = int(v >> 8), y = int(v & 0xff);
			return { { x, y, x, y } };
		}
		}
	case 4: // I
		switch (t.size)
		{
		case 0:
		{
			uint32_t v = (tm8(tm, byte_idx(t, s >> 1, tv, 0xfff)) >> ((~uint32_t(s) & 1u) * 4)) & 0xf;
			return splat4(int(v | (v << 4)));
		}
		case 1: return splat4(int(tm8(tm, byte_idx(t, s, tv, 0xfff))));
		default:
		{
			uint32_t v = tm16(tm, hw_idx(t, s, tv, 0xfff));
			int x = int(v >> 8), y = int(v & 0xff);
			return { { x, y, x, y } };
		}
		}
	default:
		return { { 0, 0, 0, 0 } };
	}
}

__device__ T4 texel_yuv(const uint16_t *tm, const RdpTile &t, int s, int tv, uint32_t chroma_x)
{
	uint32_t base = t.offset + t.stride * uint32_t(tv);
	uint32_t ol = (base + uint32_t(s)) & 0x7ff;
	uint32_t oc = (base + chroma_x * 2) & 0x7ff;
	uint32_t il = (ol ^ ((uint32_t(tv) & 1u) << 2)) ^ 3u;
	uint32_t ic = ((oc >> 1) ^ ((uint32_t(tv) & 1u) << 1)) ^ 1u;
	int luma = int(tm8(tm, il | 0x800));
	uint32_t chroma = tm16(tm, ic);
	return { { int((chroma >> 8) & 0xff) - 0x80, int(chroma & 0xff) - 0x80, luma, luma } };
}

__device__ __forceinline__ int tex_mask(int v, int mask_bits, bool mirror)
{
	if (mask_bits != 0)
	{
		int m = 1 << mask_bits;
		if (mirror) v ^= max((v & m) - 1, 0);
		v &= m - 1;
	}
	return v;
}

__device__ __forceinline__ int clamp_shift(bool clamp_bit, int coord, int lo, int hi, int shift)
{
	coord = clampi(coord, -0x8000, 0x7fff);
	if (shift < 11) coord >>= shift;
	else coord = int(unsigned(coord) << (32 - shift)) >> 16;
	if (clamp_bit)
	{
		if ((coord >> 3) >= hi) coord = (((hi >> 2) - (lo >> 2)) & 0x3ff) << 5;
		else coord = max(coord - (lo << 3), 0);
	}
	else
		coord -= lo << 3;
	return coord;
}

__device__ __forceinline__ int shift_only(int coord, int lo, int shift)
{
	coord = clampi(coord, -0x8000, 0x7fff);
	if (shift < 11) coord >>= shift;
	else coord = int(unsigned(coord) << (32 - shift)) >> 16;
	return coord - (lo << 3);
}

__device__ __forceinline__ T4 convert_factors(const T4 &in, const int16_t f[4])
{
	int x0 = bfe_s(in.v[0], 9), x1 = bfe_s(in.v[1], 9), x2 = bfe_s(in.v[2], 9);
	T4 r;
	r.v[0] = x2 + ((f[0] * x1 + 0x80) >> 8);
	r.v[1] = x2 + ((f[1] * x0 + f[2] * x1 + 0x80) >> 8);
	r.v[2] = x2 + ((f[3] * x0 + 0x80) >> 8);
	r.v[3] = x2;
	return r;
}

// texture.h:498-923
__device__ __forceinline__ T4 sample_texture(const uint16_t *tm, const RdpTile &t, int s_in, int t_in, bool tlut, bool tlut_type,
                             bool sample_quad, bool mid_state, bool convert_one, bool bilerp, const int16_t *factors,
                             const T4 &prev)
{
	int st0 = clamp_shift((t.flags & TIF_CLAMP_S) != 0, s_in, int(t.slo), int(t.shi), t.shift_s);
	int st1 = clamp_shift((t.flags & TIF_CLAMP_T) != 0, t_in, int(t.tlo), int(t.thi), t.shift_t);
	int fx = 0, fy = 0;
	if (sample_quad || tlut) { fx = st0 & 31; fy = st1 & 31; }
	int sum_frac = fx + fy;
	st0 >>= 5;
	st1 >>= 5;
	bool ms = (t.flags & TIF_MIRROR_S) != 0, mt = (t.flags & TIF_MIRROR_T) != 0;
	int s0 = tex_mask(st0, t.mask_s, ms), t0 = tex_mask(st1, t.mask_t, mt);
	int s1 = tex_mask(st0 + 1, t.mask_s, ms), t1 = tex_mask(st1 + 1, t.mask_t, mt);
	int tdiff = max(t1 - t0, -255);
	t1 = (t0 & 0xff) + tdiff;
	t0 &= 0xff;

	T4 tb = { { 0, 0, 0, 0 } }, t10 = tb, t01 = tb, t11 = tb;
	bool mid = mid_state && bilerp && fx == 0x10 && fy == 0x10;
	bool upper_lut = sum_frac >= 0x20;
	if (mid) sum_frac = 0;
	bool yuv = t.fmt == 1;
	int bs = sum_frac >= 0x20 ? s1 : s0;
	int bt = sum_frac >= 0x20 ? t1 : t0;
	int chroma_frac = ((s0 & 1) << 4) | (fx >> 1);

	if (tlut)
	{
		if (!sample_quad) { bs = s0; bt = t0; s1 = s0; t1 = t0; }
		if (t.fmt != 1)
		{
			bool upper = sum_frac >= 0x20;
			uint32_t ax = upper_lut ? 2 : 1;
			tb = fetch_texel(tm, t, bs, bt, true, tlut_type, upper ? 3 : 0, ax);
			if (bilerp)
			{
				t10 = fetch_texel(tm, t, s1, t0, true, tlut_type, 1, ax);
				t01 = fetch_texel(tm, t, s0, t1, true, tlut_type, 2, ax);
			}
			if (mid) t11 = fetch_texel(tm, t, s1, t1, true, tlut_type, 3, ax);
		}
	}
	else if (yuv)
	{
		uint32_t cx0 = uint32_t(s0 >> 1), cx1 = uint32_t((s1 + (s1 - s0)) >> 1);
		tb = texel_yuv(tm, t, s0, t0, cx0);
		if (sample_quad)
		{
			t10 = texel_yuv(tm, t, s1, t0, cx1);
			t01 = texel_yuv(tm, t, s0, t1, cx0);
			t11 = texel_yuv(tm, t, s1, t1, cx1);
		}
	}
	else if (t.fmt <= 4)
	{
		tb = fetch_texel(tm, t, bs, bt, false, false, 0, 0);
		if (sample_quad)
		{
			t10 = fetch_texel(tm, t, s1, t0, false, false, 0, 0);
			t01 = fetch_texel(tm, t, s0, t1, false, false, 0, 0);
		}
		if (mid) t11 = fetch_texel(tm, t, s1, t1, false, false, 0, 0);
	}

	T4 acc;
	if (convert_one)
	{
		int ps[4];
#pragma unroll
		for (int i = 0; i < 4; i++) ps[i] = bfe_s(prev.v[i], 9);
		if (sample_quad)
		{
			bool mid_rg = yuv ? (mid_state && chroma_frac == 0x10 && fy == 0x10) : mid;
			bool mid_ba = mid;
			bool upper_ba = sum_frac >= 32;
			bool upper_rg = yuv ? ((chroma_frac + fy) >= 32 && !mid_rg) : upper_ba;
			int frg0 = upper_rg ? ps[1] : ps[0], frg1 = upper_rg ? ps[0] : ps[1];
			int fba0 = upper_ba ? ps[1] : ps[0], fba1 = upper_ba ? ps[0] : ps[1];
#pragma unroll
			for (int i = 0; i < 4; i++)
			{
				bool m = i < 2 ? mid_rg : mid_ba;
				bool up = i < 2 ? upper_rg : upper_ba;
				int f0 = i < 2 ? frg0 : fba0, f1 = i < 2 ? frg1 : fba1;
				int cv;
				if (m)
					cv = f0 * (t01.v[i] - t11.v[i]) + f1 * (t10.v[i] - t11.v[i]) + ((tb.v[i] - t11.v[i]) << 6) + 0x80;
				else
				{
					int base = (up && yuv) ? t11.v[i] : tb.v[i];
					cv = f0 * (t10.v[i] - base) + f1 * (t01.v[i] - base) + 0x80;
				}
				acc.v[i] = (cv >> 8) + ps[2];
			}
		}
		else
			acc = splat4(ps[2]);
	}
	else if (yuv)
	{
		if (sample_quad)
		{
			int ch[2], lu[2];
			if (bilerp)
			{
				bool mid_chroma = mid_state && chroma_frac == 0x10 && fy == 0x10;
				for (int i = 0; i < 2; i++)
				{
					if (mid_chroma) ch[i] = (tb.v[i] + t10.v[i] + t11.v[i] + t01.v[i] + 2) >> 2;
					else
					{
						int sum = chroma_frac + fy;
						int base = sum >= 32 ? t11.v[i] : tb.v[i];
						int ffx = sum >= 32 ? 32 - fy : chroma_frac, ffy = sum >= 32 ? 32 - chroma_frac : fy;
						ch[i] = (((t10.v[i] - base) * ffx + (t01.v[i] - base) * ffy + 0x10) >> 5) + base;
					}
					if (mid) lu[i] = (tb.v[2 + i] + t10.v[2 + i] + t11.v[2 + i] + t01.v[2 + i] + 2) >> 2;
					else
					{
						int sum = fx + fy;
						int base = sum >= 32 ? t11.v[2 + i] : tb.v[2 + i];
						int ffx = sum >= 32 ? 32 - fy : fx, ffy = sum >= 32 ? 32 - fx : fy;
						lu[i] = (((t10.v[2 + i] - base) * ffx + (t01.v[2 + i] - base) * ffy + 0x10) >> 5) + base;
					}
				}
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
	else if (mid)
	{
#pragma unroll
		for (int i = 0; i < 4; i++) acc.v[i] = (tb.v[i] + t01.v[i] + t10.v[i] + t11.v[i] + 2) >> 2;
	}
	else if (bilerp && (sample_quad || tlut))
	{
		int ffx = sum_frac >= 32 ? 32 - fy : fx;
		int ffy = sum_frac >= 32 ? 32 - fx : fy;
#pragma unroll
		for (int i = 0; i < 4; i++)
			acc.v[i] = (((t10.v[i] - tb.v[i]) * ffx + (t01.v[i] - tb.v[i]) * ffy + 0x10) >> 5) + tb.v[i];
	}
	else
		acc = tb;

	if (!bilerp && !convert_one) acc = convert_factors(acc, factors);
	return acc;
}

// texture.h:361-472 (copy pipe)
__device__ int copy_word(const uint16_t *tm, const RdpTile &t, int st0, int st1, int s_offset, bool tlut)
{
	bool replicate = s_offset < 2 && t.size != 2 && !tlut;
	int s_shamt = min(int(t.size), 2);
	uint32_t idx_mask = (t.size == 3 || tlut) ? 0x3ffu : 0x7ffu;
	bool ms = (t.flags & TIF_MIRROR_S) != 0, mt = (t.flags & TIF_MIRROR_T) != 0;
	int samp;
	if (replicate)
	{
		st0 += 2 * s_offset;
		int sa = tex_mask(st0, t.mask_s, ms), sbv = tex_mask(st0 + 1, t.mask_s, ms);
		int tv = tex_mask(st1, t.mask_t, mt);
		uint32_t tbase = t.offset + t.stride * uint32_t(tv);
		uint32_t na = ((tbase * 2 + (uint32_t(sa) << s_shamt)) & 0x1fffu) ^ ((uint32_t(tv) & 1u) * 8u);
		uint32_t nb = ((tbase * 2 + (uint32_t(sbv) << s_shamt)) & 0x1fffu) ^ ((uint32_t(tv) & 1u) * 8u);
		int v0 = int(tm16(tm, ((na >> 2) & idx_mask) ^ 1));
		int v1 = int(tm16(tm, ((nb >> 2) & idx_mask) ^ 1));
		if (t.size == 1)
		{
			v0 = (v0 >> (8 - 4 * int(na & 2))) & 0xff;
			v1 = (v1 >> (8 - 4 * int(nb & 2))) & 0xff;
		}
		else if (t.size == 0)
		{
			v0 = ((v0 >> (12 - 4 * int(na & 3u))) & 0xf) * 0x11;
			v1 = ((v1 >> (12 - 4 * int(nb & 3u))) & 0xf) * 0x11;
		}
		else
		{
			v0 >>= 8;
			v1 >>= 8;
		}
		samp = (v0 << 8) | v1;
	}
	else
	{
		st0 += s_offset;
		int s = tex_mask(st0, t.mask_s, ms);
		int tv = tex_mask(st1, t.mask_t, mt);
		uint32_t tbase = t.offset + t.stride * uint32_t(tv);
		uint32_t nib = ((tbase * 2 + (uint32_t(s) << s_shamt)) & 0x1fffu) ^ ((uint32_t(tv) & 1u) * 8u);
		samp = int(tm16(tm, ((nib >> 2) & idx_mask) ^ 1));
		if (tlut)
		{
			if (t.size == 0)
			{
				samp = (samp >> (12 - 4 * int(nib & 3))) & 0xf;
				samp |= int(t.palette) << 4;
			}
			else
				samp = (samp >> (8 - 4 * int(nib & 2))) & 0xff;
			samp = (samp << 2) + s_offset;
			samp = int(tm16(tm, (uint32_t(samp) | 0x400u) ^ 1u));
		}
	}
	return samp;
}

// ---------------------------------------------------------------------------- combiner (combiner.h)
struct CombIn
{
	const uint8_t *cma, *cms, *cmu, *cad;
	int shade[4], comb[4], tex0[4], tex1[4];
	int lod_frac, noise;
};

__device__ __forceinline__ void pick3(int v[3], const int *src) { v[0] = src[0]; v[1] = src[1]; v[2] = src[2]; }
__device__ __forceinline__ void pick3(int v[3], const uint8_t *src) { v[0] = src[0]; v[1] = src[1]; v[2] = src[2]; }
__device__ __forceinline__ void splat3(int v[3], int x) { v[0] = v[1] = v[2] = x; }

// One combiner cycle, (A - B) * C + D per channel (combiner.h:196-282).  The selectors are the
// same for the three colour channels, so each is decoded once for all three.
__device__ __forceinline__ void combine(const CombIn &in, const uint8_t *rs, const uint8_t *as, int out[4])
{
	int a[3], b[3], m[3], d[3];
	switch (rs[0])
	{
	case 0: pick3(a, in.comb); break;
	case 1: pick3(a, in.tex0); break;
	case 2: pick3(a, in.tex1); break;
	case 4: pick3(a, in.shade); break;
	case 7: splat3(a, in.noise); break;
	case 6: splat3(a, 0x100); break;
	default: pick3(a, in.cma); break;
	}
	switch (rs[1])
	{
	case 0: pick3(b, in.comb); break;
	case 1: pick3(b, in.tex0); break;
	case 2: pick3(b, in.tex1); break;
	case 4: pick3(b, in.shade); break;
	case 7: splat3(b, (int(in.cms[1]) << 8) | in.cms[2]); break;
	default: pick3(b, in.cms); break;
	}
	switch (rs[2])
	{
	case 0: pick3(m, in.comb); break;
	case 7: splat3(m, in.comb[3]); break;
	case 1: pick3(m, in.tex0); break;
	case 2: pick3(m, in.tex1); break;
	case 4: pick3(m, in.shade); break;
	case 8: splat3(m, in.tex0[3]); break;
	case 9: splat3(m, in.tex1[3]); break;
	case 11: splat3(m, in.shade[3]); break;
	case 13: splat3(m, in.lod_frac); break;
	case 15: splat3(m, (int(in.cmu[1]) << 8) | in.cmu[2]); break;
	default: pick3(m, in.cmu); break;
	}
	switch (rs[3])
	{
	case 0: pick3(d, in.comb); break;
	case 1: pick3(d, in.tex0); break;
	case 2: pick3(d, in.tex1); break;
	case 4: pick3(d, in.shade); break;
	case 6: splat3(d, 0x100); break;
	default: pick3(d, in.cad); break;
	}
#pragma unroll
	for (int c = 0; c < 3; c++)
	{
		int col = (special_expand(a[c]) - special_expand(b[c])) * bfe_s(m[c], 9);
		col += 0x80;
		out[c] = (col >> 8) + special_expand(d[c]);
	}
	int aa, ab, am, ad;
	switch (as[0])
	{
	case 0: aa = in.comb[3]; break;
	case 1: aa = in.tex0[3]; break;
	case 2: aa = in.tex1[3]; break;
	case 4: aa = in.shade[3]; break;
	case 6: aa = 0x100; break;
	default: aa = in.cma[3]; break;
	}
	switch (as[1])
	{
	case 0: ab = in.comb[3]; break;
	case 1: ab = in.tex0[3]; break;
	case 2: ab = in.tex1[3]; break;
	case 4: ab = in.shade[3]; break;
	case 6: ab = 0x100; break;
	default: ab = in.cms[3]; break;
	}
	switch (as[2])
	{
	case 0: am = in.lod_frac; break;
	case 1: am = in.tex0[3]; break;
	case 2: am = in.tex1[3]; break;
	case 4: am = in.shade[3]; break;
	default: am = in.cmu[3]; break;
	}
	switch (as[3])
	{
	case 0: ad = in.comb[3]; break;
	case 1: ad = in.tex0[3]; break;
	case 2: ad = in.tex1[3]; break;
	case 4: ad = in.shade[3]; break;
	case 6: ad = 0x100; break;
	default: ad = in.cad[3]; break;
	}
	int col = (special_expand(aa) - special_expand(ab)) * bfe_s(am, 9);
	col += 0x80;
	out[3] = (col >> 8) + special_expand(ad);
}

// ---------------------------------------------------------------------------- z encode / depth test / blender
__device__ __forceinline__ int z_decompress(int z)
{
	int e = z >> 11, m = z & 0x7ff;
	return (m << max(6 - e, 0)) + (0x40000 - (0x40000 >> e));
}
__device__ __forceinline__ int z_compress(int z)
{
	int inv = max(0x3ffff - z, 1);
	int e = clampi(17 - find_msb(inv), 0, 7);
	int m = (z >> max(6 - e, 0)) & 0x7ff;
	return ((e << 11) + m) & 0xffff;
}

struct Pix
{
	int col[4];
	int depth, dz;
	bool cdirty, ddirty;
	uint32_t cidx;
};

__device__ __forceinline__ void blender(const int pix[4], const int mem[4], const uint8_t fog[4], const uint8_t bc[4], int shade_alpha,
                        const uint8_t *m, bool force_blend, bool blend_en, bool color_on_cvg, bool cvg_wrap,
                        const int bshift[2], bool final_cycle, int out[3])
{
	// Each selector decoded once for the three channels.
	int r1[3], r0[3];
	switch (m[2])
	{
	case 0: pick3(r1, pix); break;
	case 1: pick3(r1, mem); break;
	case 2: pick3(r1, bc); break;
	default: pick3(r1, fog); break;
	}
	switch (m[0])
	{
	case 0: pick3(r0, pix); break;
	case 1: pick3(r0, mem); break;
	case 2: pick3(r0, bc); break;
	default: pick3(r0, fog); break;
	}
	if (final_cycle && color_on_cvg && !cvg_wrap)
	{
		out[0] = r1[0]; out[1] = r1[1]; out[2] = r1[2];
		return;
	}
	if (final_cycle && (!blend_en || (m[1] == 0 && m[3] == 0 && pix[3] == 0xff)))
	{
		out[0] = r0[0]; out[1] = r0[1]; out[2] = r0[2];
		return;
	}
	int a0, a1;
	switch (m[1])
	{
	case 0: a0 = pix[3]; break;
	case 1: a0 = fog[3]; break;
	case 2: a0 = shade_alpha; break;
	default: a0 = 0; break;
	}
	switch (m[3])
	{
	case 0: a1 = ~a0 & 0xff; break;
	case 1: a1 = mem[3]; break;
	case 2: a1 = 0xff; break;
	default: a1 = 0; break;
	}
	a0 >>= 3;
	a1 >>= 3;
	if (m[3] == 1)
	{
		a0 = (a0 >> bshift[0]) & 0x3c;
		a1 = (a1 >> bshift[1]) | 3;
	}
	if (!final_cycle || force_blend)
	{
#pragma unroll
		for (int c = 0; c < 3; c++) out[c] = ((r0[c] * a0 + r1[c] * (a1 + 1)) >> 5) & 0xff;
	}
	else
	{
		int sum = (a0 >> 2) + (a1 >> 2) + 1;
#pragma unroll
		for (int c = 0; c < 3; c++)
		{
			int v = ((r0[c] * a0 + r1[c] * (a1 + 1)) >> 2) & 0x7ff;
			out[c] = g_blender_lut[((sum << 11) | v) & 0x7fff];
		}
	}
}

// ---------------------------------------------------------------------------- RDRAM framebuffer I/O
__device__ __forceinline__ uint16_t ld16(const RdpPass &p, uint32_t i)
{
	return *reinterpret_cast<const uint16_t *>(p.rdram + ((i * 2) & (p.rdram_size - 1)));
}
__device__ __forceinline__ void st16(const RdpPass &p, uint32_t i, uint16_t v)
{
	*reinterpret_cast<uint16_t *>(p.rdram + ((i * 2) & (p.rdram_size - 1))) = v;
}
__device__ __forceinline__ uint8_t hid(const RdpPass &p, uint32_t i) { return p.hidden[i & (p.hidden_size - 1)]; }
__device__ __forceinline__ void whid(const RdpPass &p, uint32_t i, uint8_t v) { p.hidden[i & (p.hidden_size - 1)] = v; }

__device__ void load_pixel(const RdpPass &p, Pix &px, uint32_t ci, uint32_t di)
{
	px.cidx = ci;
	px.cdirty = px.ddirty = false;
	switch (p.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8:
	{
		uint32_t idx = ci & (p.rdram_size - 1);
		int w = p.rdram[idx ^ 3u];
		px.col[0] = px.col[1] = px.col[2] = w;
		px.col[3] = hid(p, idx >> 1);
		break;
	}
	case FBF_RGBA5551:
	{
		uint32_t idx = ci & ((p.rdram_size >> 1) - 1);
		uint32_t w = ld16(p, idx ^ 1u);
		px.col[0] = int((w >> 8) & 0xf8u);
		px.col[1] = int((w >> 3) & 0xf8u);
		px.col[2] = int((w << 2) & 0xf8u);
		px.col[3] = ((hid(p, idx) << 5) | int((w & 1) << 7)) & 0xff;
		break;
	}
	case FBF_IA88:
	{
		uint32_t idx = ci & ((p.rdram_size >> 1) - 1);
		uint32_t w = ld16(p, idx ^ 1u);
		px.col[0] = px.col[1] = px.col[2] = int((w >> 8) & 0xff);
		px.col[3] = int(w & 0xff);
		break;
	}
	default:
	{
		uint32_t idx = ci & ((p.rdram_size >> 2) - 1);
		uint32_t w = *reinterpret_cast<const uint32_t *>(p.rdram + idx * 4);
#pragma unroll
		for (int c = 0; c < 4; c++) px.col[c] = int((w >> (24 - 8 * c)) & 0xff);
		break;
	}
	}
	uint32_t didx = di & ((p.rdram_size >> 1) - 1);
	uint32_t w = ld16(p, didx ^ 1u);
	px.depth = int(w >> 2);
	px.dz = (hid(p, didx) | int((w & 3) << 2)) & 0xff;
}

// Marks RDRAM bytes [addr, addr + n) (n <= 4, not crossing a 32-byte line: the pixel formats'
// natural alignment) as written by the GPU in the instance's write mask, which the masked
// write-back to the caller's RDRAM reads.  Called by all 32 lanes of a warp together; lanes whose
// bytes share a mask word merge them into one atomic.
__device__ __forceinline__ void mark_written(const RdpPass &p, bool any, uint32_t addr, uint32_t n)
{
	if (!p.wmask) return;
	const uint32_t word = any ? (addr & (p.rdram_size - 1)) >> 5 : 0xffffffffu;
	const uint32_t bits = any ? ((n >= 32 ? 0xffffffffu : ((1u << n) - 1u)) << (addr & 31u)) : 0u;
	const unsigned peers = __match_any_sync(0xffffffffu, word);
	const uint32_t merged = __reduce_or_sync(peers, bits);
	if (any && (__ffs(int(peers)) - 1) == int(threadIdx.x & 31)) atomicOr(p.wmask + word, merged);
}

// The bytes a pixel store writes: colour (1, 2 or 4 bytes at the format's address swizzle) and depth
// (2 bytes).  Mirrors store_pixel's addressing.
__device__ __forceinline__ void mark_pixel(const RdpPass &p, const Pix &px, uint32_t ci, uint32_t di, bool alias,
                                           bool stored)
{
	bool c = stored && px.cdirty, d = stored && !alias && px.ddirty;
	uint32_t ca = 0, cn = 0;
	switch (p.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8: ca = (ci & (p.rdram_size - 1)) ^ 3u; cn = 1; break;
	case FBF_RGBA5551:
	case FBF_IA88: ca = ((ci & ((p.rdram_size >> 1) - 1)) ^ 1u) * 2u; cn = 2; break;
	default: ca = (ci & ((p.rdram_size >> 2) - 1)) * 4u; cn = 4; break;
	}
	mark_written(p, c, ca, cn);
	mark_written(p, d, ((di & ((p.rdram_size >> 1) - 1)) ^ 1u) * 2u, 2);
}

__device__ void store_pixel(const RdpPass &p, const Pix &px, uint32_t ci, uint32_t di, bool alias)
{
	if (px.cdirty)
	{
		switch (p.fb_fmt)
		{
		case FBF_I4:
		{
			uint32_t idx = ci & (p.rdram_size - 1);
			p.rdram[idx ^ 3u] = 0;
			if (idx & 1u) whid(p, idx >> 1, uint8_t(px.col[3]));
			break;
		}
		case FBF_I8:
		{
			uint32_t idx = ci & (p.rdram_size - 1);
			uint32_t col = (idx & 1) ? uint32_t(px.col[1]) : uint32_t(px.col[0]);
			p.rdram[idx ^ 3u] = uint8_t(col);
			if (idx & 1u) whid(p, idx >> 1, uint8_t((col & 1) * 3));
			break;
		}
		case FBF_RGBA5551:
		{
			uint32_t idx = ci & ((p.rdram_size >> 1) - 1);
			uint32_t cov = uint32_t(px.col[3]) >> 5;
			uint32_t w = ((uint32_t(px.col[0]) & 0xf8u) << 8) | ((uint32_t(px.col[1]) & 0xf8u) << 3) |
			             ((uint32_t(px.col[2]) & 0xf8u) >> 2) | (cov >> 2);
			st16(p, idx ^ 1u, uint16_t(w));
			whid(p, idx, uint8_t(cov & 3u));
			break;
		}
		case FBF_IA88:
		{
			uint32_t idx = ci & ((p.rdram_size >> 1) - 1);
			st16(p, idx ^ 1u, uint16_t((uint32_t(px.col[0]) << 8) | uint32_t(px.col[3])));
			whid(p, idx, uint8_t((px.col[3] & 1) * 3));
			break;
		}
		default:
		{
			uint32_t idx = ci & ((p.rdram_size >> 2) - 1);
			uint32_t w = (uint32_t(px.col[0]) << 24) | (uint32_t(px.col[1]) << 16) | (uint32_t(px.col[2]) << 8) |
			             uint32_t(px.col[3]);
			*reinterpret_cast<uint32_t *>(p.rdram + idx * 4) = w;
			whid(p, 2u * idx, uint8_t((px.col[1] & 1) * 3));
			whid(p, 2u * idx + 1u, uint8_t((px.col[3] & 1) * 3));
			break;
		}
		}
	}
	if (!alias && px.ddirty)
	{
		uint32_t idx = di & ((p.rdram_size >> 1) - 1);
		st16(p, idx ^ 1u, uint16_t((px.depth << 2) | (px.dz >> 2)));
		whid(p, idx, uint8_t(px.dz & 3));
	}
}

__device__ void alias_c2d(uint32_t fmt, Pix &px)
{
	if (fmt == FBF_RGBA5551)
	{
		px.dz = ((px.col[3] >> 3) | (px.col[2] & 8)) & 0xff;
		uint32_t w = ((uint32_t(px.col[0]) & 0xf8u) << 6) | ((uint32_t(px.col[1]) & 0xf8u) << 1) |
		             ((uint32_t(px.col[2]) & 0xf8u) >> 4);
		px.depth = int(w & 0xffff);
	}
	else if (fmt == FBF_IA88)
	{
		uint32_t w = (uint32_t(px.col[0]) << 8) | uint32_t(px.col[3]);
		px.depth = int((w >> 2) & 0xffff);
		px.dz = int((((w & 3u) << 2) | ((w & 1u) * 3u)) & 0xff);
	}
}

__device__ void alias_d2c(uint32_t fmt, Pix &px)
{
	uint32_t w = (uint32_t(px.depth) << 4) | uint32_t(px.dz);
	if (fmt == FBF_RGBA5551)
	{
		px.col[0] = int((w >> 10) & 0xf8u);
		px.col[1] = int((w >> 5) & 0xf8u);
		px.col[2] = int(w & 0xf8u);
		px.col[3] = int((w & 7u) << 5);
	}
	else if (fmt == FBF_IA88)
	{
		px.col[0] = int((w >> 10) & 0xffu);
		px.col[3] = int((w >> 2) & 0xffu);
	}
	px.cdirty = true;
}

__device__ __forceinline__ void write_color(uint32_t fmt, Pix &px, int r, int g, int b, int a)
{
	px.col[0] = r; px.col[1] = g; px.col[2] = b;
	if (fmt != FBF_I4) px.col[3] = a;
	px.cdirty = true;
}

// ---------------------------------------------------------------------------- per pixel: shade + blend
// RGB dither value of a pixel (dither.h:39-58): a cell of the magic-square or Bayer matrix
// replicated over the three channels, the low 9 bits of the pixel's noise, or none.
__device__ __forceinline__ int rgb_dither_value(uint32_t static_flags, uint32_t dither, int x, int y, uint32_t noise)
{
	const int yy = y >> int((static_flags & RS_INTERLACE_FIELD) != 0);
	const int mr = int(dither >> 2), cell = (yy & 3) * 4 + (x & 3);
	if (mr < 2) return g_dither[mr][cell] * (1 | 8 | 64);
	if (mr == 2) return int(noise & 0x1ffu);
	return 0;
}

// Shaded record of one pixel in the shading scratch (8 bytes): x = combined RGBA; y = z (18
// bits; the copy pipe's texel word, 16 bits) | code << 18 | shade alpha << 22, code = coverage
// 0-8, SC_COPY, SC_FILL or SC_NONE (not written).  The RGB dither bits are not stored: k_blend
// recomputes them from the pixel and the primitive (rgb_dither_value).
constexpr uint32_t SC_COPY = 9, SC_FILL = 10, SC_NONE = 15;
constexpr uint2 kScratchEmpty = { 0u, 0xffffffffu };

struct PassConst
{
	int fb_size, dx_mask, dx_shift;
	bool alias;
	int sl = 0; // log2 of the upscaling factor: 0 for every pass but an upscaled one
};

// Output of the shading stage for one pixel and primitive (the reference's ShadedData,
// data_structures.h:319-325): coverage 0..8, or COPY (0x20) / FILL (0x40) flags.
struct Shaded
{
	uint32_t combined; // r | g << 8 | b << 16 | a << 24
	int z_dith;        // z << 9 | rgb dither, or the copy-pipe texel word
	int coverage;
	int shade_alpha;
};

// shading.h:38-359: everything that does not depend on the framebuffer.
//
// Specialised per static render state (the reference compiles its shading shaders per
// normalised static state with specialisation constants, rdp_renderer.cpp:1294-1331,
// 1790-1822): the static flags in KN are known at compile time to equal KV's, so every branch on
// them folds away; the other flags are read at run time.  KN = 0 is the general shader.
template <uint32_t KN, uint32_t KV>
__device__ __forceinline__ bool shade_pixel_v(const PassConst &pc, const RdpPrimGeom &g, const RdpPrimAttr &a,
                                              const RdpPrimShade &sh, const RdpTile *tiles, const uint16_t *tm,
                                              const SpanRow &sp, const SpanRow &sp_next, int x, int y, Shaded &out)
{
	if (!sp.valid) return false;
	const uint32_t f = sh.static_flags;
#define F(bit) ((KN & (bit)) ? ((KV & (bit)) != 0) : ((f & (bit)) != 0))
	const bool flip = (g.flags & TRI_FLIP) != 0;
	const bool perspective = F(RS_PERSPECTIVE);
	uint32_t noise = 0;
	if (F(RS_NEED_NOISE)) noise = reseed_noise(uint32_t(x), uint32_t(y), sh.prim_index);

	if (F(RS_COPY))
	{
		if (!(x >= sp.start_x && x <= sp.end_x)) return false;
		int dxp = flip ? (x - sp.start_x) : (sp.end_x - x);
		dxp >>= pc.sl; // upscaled copies repeat pixels (interpolation.h:60-61)
		int s_offset = dxp - (dxp & pc.dx_mask);
		int lerp_dx = (dxp >> pc.dx_shift) * (flip ? 1 : -1);
		int s = (sp.stzw[0] + mulw(a.dstzw_dx[0] & ~0x1f, lerp_dx)) >> 16;
		int t = (sp.stzw[1] + mulw(a.dstzw_dx[1] & ~0x1f, lerp_dx)) >> 16;
		int w = (sp.stzw[3] + mulw(a.dstzw_dx[3] & ~0x1f, lerp_dx)) >> 16;
		int os, ot;
		bool ov = false;
		st_div(s, t, w, perspective, os, ot, ov);
		const RdpTile &t0 = tiles[g.tile & 7];
		int st0 = shift_only(os, int(t0.slo), t0.shift_s) >> 5;
		int st1 = shift_only(ot, int(t0.tlo), t0.shift_t) >> 5;
		bool tlut = F(RS_TLUT);
		int texel;
		if (pc.fb_size == 0) texel = 0;
		else if (pc.fb_size == 1)
			texel = (copy_word(tm, t0, st0, st1, s_offset >> 1, tlut) >> (8 - 8 * (s_offset & 1))) & 0xff;
		else
			texel = copy_word(tm, t0, st0, st1, s_offset, tlut);
		if (F(RS_ALPHA_TEST) && pc.fb_size == 2 && (texel & 1) == 0) return false;
		out.z_dith = texel;
		out.coverage = 0x20;
		return true;
	}
	if (F(RS_FILL))
	{
		out.coverage = 0x40;
		return x >= sp.start_x && x <= sp.end_x;
	}

	// ---- coverage (coverage.h:31-47)
	int coverage;
	{
		int xs = x << 3;
		int clip = 0;
#pragma unroll
		for (int k = 0; k < 4; k++)
		{
			int off = (k == 0) ? 0 : (k == 1 ? 4 : (k == 2 ? 2 : 6));
			int xsh = xs + off;
			int l0 = k >> 1, l1 = 2 + (k >> 1);
			if (xsh < sp.xl[l0] || xsh >= sp.xr[l0]) clip |= 1 << k;
			if (xsh < sp.xl[l1] || xsh >= sp.xr[l1]) clip |= 16 << k;
		}
		coverage = ~clip & 0xff;
	}
	if (coverage == 0) return false;
	int cov_count = __popc(coverage);
	const bool aa = F(RS_AA);
	if (!aa && (coverage & 1) == 0) return false;

	int dx = x - sp.base_x;
	int idir = flip ? 1 : -1;
	int first = find_lsb(unsigned(coverage));
	int yoff = first >> 1;
	int xoff = ((first & 1) << 1) + (yoff & 1);

	// ---- interpolate_rgba (interpolation.h:30-51)
	const int sl = pc.sl;
	int shade[4];
#pragma unroll
	for (int c = 0; c < 4; c++)
	{
		int v = sp.rgba[c] + mulw((a.drgba_dx[c] & ~0x1f) >> sl, dx);
		int sn = shlw(v >> 14, 2 + sl);
		sn += xoff * (a.drgba_dx[c] >> 14) + yoff * (a.drgba_dy[c] >> 14);
		sn >>= 4 + sl;
		shade[c] = clamp_9bit(sn);
	}

	// ---- interpolate_stz (interpolation.h:92-142)
	const bool uses_lod = F(RS_USES_LOD);
	int s0 = 0, t0v = 0, sdx = 0, tdx = 0, sdy = 0, tdy = 0, z;
	bool povf = false;
	{
		int sw[3], idx3[3] = { 0, 1, 3 };
#pragma unroll
		for (int k = 0; k < 3; k++) sw[k] = sp.stzw[idx3[k]] + mulw((a.dstzw_dx[idx3[k]] & ~0x1f) >> sl, dx);
		if (F(RS_USES_TEXEL0) || F(RS_USES_TEXEL1) || F(RS_USES_PIPELINED_TEXEL1) || F(RS_USES_LOD))
		{
			st_div(sw[0] >> 16, sw[1] >> 16, sw[2] >> 16, perspective, s0, t0v, povf);
			if (uses_lod)
			{
				// Upscaled: the LOD step in x covers one native pixel with native_texture_lod, and
				// the y step scales the same way (interpolation.h:100-108, shading.h:193-196).
				const int tdir = (sl && (g.flags & TRI_NATIVE_LOD)) ? (idir << sl) : idir;
				const int ymul = sl ? abs(tdir) : 1;
				int wx[3], wy[3];
#pragma unroll
				for (int k = 0; k < 3; k++)
				{
					wx[k] = sw[k] + mulw(tdir, (a.dstzw_dx[idx3[k]] & ~0x1f) >> sl);
					wy[k] = sw[k] + mulw(ymul, (a.dstzw_dy[idx3[k]] & ~0x7fff) >> sl);
				}
				st_div(wx[0] >> 16, wx[1] >> 16, wx[2] >> 16, perspective, sdx, tdx, povf);
				st_div(wy[0] >> 16, wy[1] >> 16, wy[2] >> 16, perspective, sdy, tdy, povf);
			}
		}
		z = sp.stzw[2] + mulw(a.dstzw_dx[2], dx >> sl) + mulw(a.dstzw_dx[2] >> sl, dx & ((1 << sl) - 1));
		int sz = shlw(z >> 10, 2 + sl);
		sz += xoff * (a.dstzw_dx[2] >> 10) + yoff * (a.dstzw_dy[2] >> 10);
		sz >>= 5 + sl;
		z = clamp_z(sz);
	}

	// ---- LOD (texture.h:925-1003)
	uint32_t tile0 = g.tile & 7u, tile1 = (tile0 + 1) & 7u, max_level = g.tile >> 3;
	int lod_frac = 0;
	if (uses_lod)
	{
		bool sharpen = F(RS_SHARPEN), detail = F(RS_DETAIL);
		bool magnify = false, distant = false;
		uint32_t tofs = 0;
		if (povf)
		{
			distant = true;
			lod_frac = 0xff;
		}
		else
		{
			int dxs = sdx - s0, dxt = tdx - t0v, dys = sdy - s0, dyt = tdy - t0v;
			dxs ^= dxs >> 31; dxt ^= dxt >> 31; dys ^= dys >> 31; dyt ^= dyt >> 31;
			int max_d = max(max(dxs, dys), max(dxt, dyt));
			if (max_d >= 0x4000)
			{
				distant = true;
				lod_frac = 0xff;
				tofs = max_level;
			}
			else if (max_d < 32)
			{
				distant = max_level == 0u;
				magnify = true;
				if (!sharpen && !detail) lod_frac = distant ? 0xff : 0;
				else lod_frac = (max(int(sh.min_lod), max_d) << 3) + (sharpen ? -0x100 : 0);
			}
			else
			{
				int mip_base = max(find_msb(max_d >> 5), 0);
				distant = uint32_t(mip_base) >= max_level;
				if (distant && !sharpen && !detail) lod_frac = 0xff;
				else
				{
					lod_frac = ((max_d << 3) >> mip_base) & 0xff;
					tofs = uint32_t(mip_base);
				}
			}
		}
		if (F(RS_TEX_LOD))
		{
			if (distant) tofs = max_level;
			if (!detail)
			{
				tile0 = (tile0 + tofs) & 7u;
				tile1 = (distant || (!sharpen && magnify)) ? tile0 : ((tile0 + 1) & 7u);
			}
			else
			{
				tile1 = (tile0 + tofs + ((distant || magnify) ? 1 : 2)) & 7u;
				tile0 = (tile0 + tofs + (magnify ? 0 : 1)) & 7u;
			}
		}
	}

	// ---- texels
	const bool tlut = F(RS_TLUT), tlut_type = F(RS_TLUT_TYPE);
	const bool quad = F(RS_SAMPLE_QUAD), midt = F(RS_MID_TEXEL);
	T4 tex0 = { { 0, 0, 0, 0 } }, tex1 = tex0;
	if (F(RS_USES_TEXEL0))
		tex0 = sample_texture(tm, tiles[tile0], s0, t0v, tlut, tlut_type, quad, midt, false, F(RS_BILERP0),
		                      sh.factors, tex0);
	bool uses_t1 = F(RS_USES_TEXEL1);
	if (F(RS_USES_PIPELINED_TEXEL1))
	{
		int lodlength = int16_t(flip ? (sp.end_x - sp.base_x) : (sp.base_x - sp.start_x));
		bool end_span = x == (flip ? sp.end_x : sp.start_x);
		if (end_span && lodlength >= 8 && sp_next.valid)
		{
			bool dummy = false;
			st_div(sp_next.stzw[0] >> 16, sp_next.stzw[1] >> 16, sp_next.stzw[3] >> 16, perspective, s0, t0v, dummy);
		}
		else
		{
			int ndx = dx + (idir << sl);
			int ss = (sp.stzw[0] + mulw((a.dstzw_dx[0] & ~0x1f) >> sl, ndx)) >> 16;
			int tt = (sp.stzw[1] + mulw((a.dstzw_dx[1] & ~0x1f) >> sl, ndx)) >> 16;
			int ww = (sp.stzw[3] + mulw((a.dstzw_dx[3] & ~0x1f) >> sl, ndx)) >> 16;
			bool dummy = false;
			st_div(ss, tt, ww, perspective, s0, t0v, dummy);
		}
		tile1 = tile0;
		uses_t1 = true;
	}
	if (uses_t1)
	{
		bool c1 = F(RS_CONVERT_ONE), b1 = F(RS_BILERP1);
		if (c1 && !b1) tex1 = convert_factors(tex0, sh.factors);
		else tex1 = sample_texture(tm, tiles[tile1], s0, t0v, tlut, tlut_type, quad, midt, c1, b1, sh.factors, tex0);
	}

	// ---- dither coefficients (dither.h:39-68)
	const int rgb_d = rgb_dither_value(f, sh.dither, x, y, noise);
	int alpha_d;
	{
		int yy = y >> int(F(RS_INTERLACE_FIELD));
		int mr = int(sh.dither >> 2), ma = int(sh.dither & 3);
		int cell = (yy & 3) * 4 + (x & 3);
		if (ma == 3) alpha_d = 0;
		else if (ma == 2) alpha_d = int(noise & 7u);
		else
		{
			alpha_d = mr >= 2 ? g_dither[mr & 1][cell] : (rgb_d & 7);
			if (ma == 1) alpha_d = ~alpha_d & 7;
		}
	}

	// ---- combiner (shading.h:263-333, combiner.h:196-282)
	const bool cvg_times_alpha = F(RS_CVG_TIMES_ALPHA), alpha_cvg_select = F(RS_ALPHA_CVG_SELECT);
	const bool alpha_test = F(RS_ALPHA_TEST);
	int combined[4];
	int alpha_ref = 0;
	CombIn in;
#pragma unroll
	for (int c = 0; c < 4; c++)
	{
		in.shade[c] = shade[c];
		in.comb[c] = 0;
		in.tex0[c] = tex0.v[c];
		in.tex1[c] = tex1.v[c];
	}
	in.lod_frac = lod_frac;
	in.noise = int(((noise & 7u) << 6) | 0x20u);
	// Cycle 0 (2-cycle mode only), then cycle 1, through one inlined copy of the combiner.
#pragma unroll 1
	for (int cy = F(RS_MULTI_CYCLE) ? 0 : 1; cy < 2; cy++)
	{
		in.cma = sh.c_muladd[cy]; in.cms = sh.c_mulsub[cy]; in.cmu = sh.c_mul[cy]; in.cad = sh.c_add[cy];
		combine(in, sh.comb_rgb[cy], sh.comb_alpha[cy], combined);
		if (cy == 0)
		{
			if (alpha_test)
			{
				int ca = clamp_9bit(combined[3]);
				int ea = ca + ((ca + 1) >> 8);
				if (alpha_cvg_select) ea = cvg_times_alpha ? ((ea * cov_count + 4) >> 3) : (cov_count << 5);
				else ea += alpha_d;
				alpha_ref = clampi(ea, 0, 0xff);
			}
#pragma unroll
			for (int c = 0; c < 4; c++)
			{
				in.comb[c] = combined[c];
				int tmp = in.tex0[c];
				in.tex0[c] = in.tex1[c];
				in.tex1[c] = tmp;
			}
			if (F(RS_NEED_NOISE_DUAL))
			{
				// The second seed also feeds the later alpha-test threshold (shading.h:309-347).
				noise = reseed_noise(uint32_t(x + 1023), uint32_t(y + 7), sh.prim_index + 11);
				in.noise = int(((noise & 7u) << 6) | 0x20u);
			}
		}
	}
	// combiner_cycle1 tail
#pragma unroll
	for (int c = 0; c < 4; c++) combined[c] = clamp_9bit(combined[c]);
	{
		int ea = combined[3] + ((combined[3] + 1) >> 8);
		int mod;
		if (cvg_times_alpha)
		{
			mod = (ea * cov_count + 4) >> 3;
			cov_count = mod >> 5;
		}
		else
			mod = cov_count << 5;
		if (alpha_cvg_select) ea = mod;
		else ea += alpha_d;
		combined[3] = clampi(ea, 0, 0xff);
	}
	if (!F(RS_MULTI_CYCLE)) alpha_ref = combined[3];
	if (aa && cov_count == 0) return false;
	if (alpha_test)
	{
		int thr = F(RS_ALPHA_TEST_DITHER) ? int(noise & 0xffu) : int(sh.blend_color[3]);
		if (alpha_ref < thr) return false;
	}

	out.combined = uint32_t(combined[0] & 0xff) | (uint32_t(combined[1] & 0xff) << 8) |
	               (uint32_t(combined[2] & 0xff) << 16) | (uint32_t(combined[3] & 0xff) << 24);
	out.z_dith = (z << 9) | rgb_d;
	out.coverage = cov_count;
	out.shade_alpha = min(shade[3] + alpha_d, 0xff);
	return true;
#undef F
}

// The general shader: every static flag read at run time.
__device__ __forceinline__ bool shade_pixel(const PassConst &pc, const RdpPrimGeom &g, const RdpPrimAttr &a,
                                            const RdpPrimShade &sh, const RdpTile *tiles, const uint16_t *tm,
                                            const SpanRow &sp, const SpanRow &sp_next, int x, int y, Shaded &out)
{
	return shade_pixel_v<0u, 0u>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
}

// Render-state variants with their own compiled shading code (the kernels' SPEC instantiations).
// A primitive takes the first variant whose known flags equal its own: (static_flags & KN) == KV;
// the rest take the general shader.  The keys are the flags that select whole paths of
// shading.h -- which pipe (fill, copy, the 1/2-cycle pipeline), which texels and LOD are used, TLUT,
// noise -- so a variant's code holds only its path.  The variants compute exactly what the
// general shader computes for the same primitive.
constexpr uint32_t SV_PIPE = RS_COPY | RS_FILL;
constexpr uint32_t SV_TEX = RS_USES_TEXEL0 | RS_USES_TEXEL1 | RS_USES_PIPELINED_TEXEL1 | RS_USES_LOD;
constexpr uint32_t SV_NOISE = RS_NEED_NOISE | RS_NEED_NOISE_DUAL;
constexpr uint32_t SV_FILL_KN = SV_PIPE, SV_FILL_KV = RS_FILL;
constexpr uint32_t SV_COPY_KN = SV_PIPE, SV_COPY_KV = RS_COPY;
constexpr uint32_t SV_FLAT_KN = SV_PIPE | SV_TEX | SV_NOISE, SV_FLAT_KV = 0;
constexpr uint32_t SV_TEX0_KN = SV_PIPE | SV_TEX | SV_NOISE | RS_TLUT | RS_CONVERT_ONE;
constexpr uint32_t SV_TEX0_KV = RS_USES_TEXEL0, SV_TLUT0_KV = RS_USES_TEXEL0 | RS_TLUT;
constexpr uint32_t SV_TEX01_KN = SV_PIPE | SV_TEX | SV_NOISE | RS_TLUT, SV_TEX01_KV = RS_USES_TEXEL0 | RS_USES_TEXEL1;
constexpr uint32_t SV_LOD_KN = SV_PIPE | RS_USES_LOD | SV_NOISE | RS_TLUT, SV_LOD_KV = RS_USES_LOD;

template <bool SPEC>
__device__ __forceinline__ bool shade_pixel_any(const PassConst &pc, const RdpPrimGeom &g, const RdpPrimAttr &a,
                                                const RdpPrimShade &sh, const RdpTile *tiles, const uint16_t *tm,
                                                const SpanRow &sp, const SpanRow &sp_next, int x, int y, Shaded &out)
{
	if (SPEC)
	{
		const uint32_t f = sh.static_flags;
		if ((f & SV_FILL_KN) == SV_FILL_KV)
			return shade_pixel_v<SV_FILL_KN, SV_FILL_KV>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
		if ((f & SV_COPY_KN) == SV_COPY_KV)
			return shade_pixel_v<SV_COPY_KN, SV_COPY_KV>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
		if ((f & SV_FLAT_KN) == SV_FLAT_KV)
			return shade_pixel_v<SV_FLAT_KN, SV_FLAT_KV>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
		if ((f & SV_TEX0_KN) == SV_TEX0_KV)
			return shade_pixel_v<SV_TEX0_KN, SV_TEX0_KV>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
		if ((f & SV_TEX0_KN) == SV_TLUT0_KV)
			return shade_pixel_v<SV_TEX0_KN, SV_TLUT0_KV>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
		if ((f & SV_TEX01_KN) == SV_TEX01_KV)
			return shade_pixel_v<SV_TEX01_KN, SV_TEX01_KV>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
		if ((f & SV_LOD_KN) == SV_LOD_KV)
			return shade_pixel_v<SV_LOD_KN, SV_LOD_KV>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
	}
	return shade_pixel_v<0u, 0u>(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out);
}

// The framebuffer half: fill pipe, copy pipe or depth test + blender + dither + coverage
// (memory_interfacing.h:381-571).  Returns whether the pixel was written.
__device__ __forceinline__ uint2 pack_shaded(const Shaded &o)
{
	uint32_t y;
	if (o.coverage & 0x40) y = SC_FILL << 18;
	else if (o.coverage & 0x20) y = (uint32_t(o.z_dith) & 0xffffu) | (SC_COPY << 18);
	else y = (uint32_t(o.z_dith) >> 9) | (uint32_t(o.coverage) << 18) | (uint32_t(o.shade_alpha) << 22);
	return make_uint2(o.combined, y);
}

// The fill pipe (memory_interfacing.h:381-571, fill branch): the pixel takes the fill colour,
// the 16-bit formats the half of the 32-bit fill word at the pixel's address.
__device__ __forceinline__ bool fill_pixel(const RdpPass &ps, const PassConst &pc, uint32_t col, Pix &px)
{
	switch (ps.fb_fmt)
	{
	case FBF_RGBA8888:
		write_color(ps.fb_fmt, px, int((col >> 24) & 0xff), int((col >> 16) & 0xff), int((col >> 8) & 0xff), int(col & 0xff));
		break;
	case FBF_RGBA5551:
		col >>= ((px.cidx & 1u) ^ 1u) * 16u;
		write_color(ps.fb_fmt, px, int((col >> 8) & 0xf8u), int((col >> 3) & 0xf8u), int((col << 2) & 0xf8u),
		            int((col & 1u) * 0xe0u));
		break;
	case FBF_IA88:
	{
		col >>= ((px.cidx & 1u) ^ 1u) * 16u;
		int r = int((col >> 8) & 0xff);
		write_color(ps.fb_fmt, px, r, r, r, int(col & 0xff));
		break;
	}
	case FBF_I8:
	{
		col >>= ((px.cidx & 3u) ^ 3u) * 8u;
		int v = int(col & 0xff);
		write_color(ps.fb_fmt, px, v, v, v, v);
		break;
	}
	default: break;
	}
	if (pc.alias) alias_c2d(ps.fb_fmt, px);
	return ps.fb_fmt != FBF_I4;
}

__device__ bool blend_pixel(const RdpPass &ps, const PassConst &pc, const RdpPrimShade &sh, const Shaded &in, Pix &px)
{
	if (in.coverage & 0x40) return fill_pixel(ps, pc, sh.fill_color, px);
	if (in.coverage & 0x20)
	{
		uint32_t word = uint32_t(in.z_dith);
		switch (ps.fb_fmt)
		{
		case FBF_I4: px.col[0] = px.col[1] = px.col[2] = px.col[3] = 0; px.cdirty = true; break;
		case FBF_I8: { int v = int(word & 0xffu); write_color(ps.fb_fmt, px, v, v, v, v); break; }
		case FBF_RGBA5551:
			write_color(ps.fb_fmt, px, int((word >> 8) & 0xf8u), int((word >> 3) & 0xf8u), int((word << 2) & 0xf8u),
			            int((word & 1) * 0xe0u));
			break;
		default: break;
		}
		if (pc.alias) alias_c2d(ps.fb_fmt, px);
		return ps.fb_fmt == FBF_I4 || ps.fb_fmt == FBF_I8 || ps.fb_fmt == FBF_RGBA5551;
	}
	const int z = in.z_dith >> 9;
	const int rgb_d = in.z_dith & 0x1ff;
	int cov_count = in.coverage;
	const int shade_alpha = in.shade_alpha;
	int combined[4] = { int(in.combined & 0xff), int((in.combined >> 8) & 0xff), int((in.combined >> 16) & 0xff),
	                    int(in.combined >> 24) };
	// ---- depth_blend (memory_interfacing.h:488-571)
	const uint32_t df = sh.db_flags;
	const bool force_blend = (df & DB_FORCE_BLEND) != 0, image_read = (df & DB_IMAGE_READ) != 0;
	const bool dba = (df & DB_AA) != 0;
	int mem[4];
	{
		int mc = image_read ? (px.col[3] & 0xe0) : 0xe0;
		switch (ps.fb_fmt)
		{
		case FBF_I4: mem[0] = mem[1] = mem[2] = 0; mc = 0xe0; break;
		case FBF_I8: mem[0] = mem[1] = mem[2] = px.col[0]; mc = 0xe0; break;
		case FBF_RGBA5551: mem[0] = px.col[0] & 0xf8; mem[1] = px.col[1] & 0xf8; mem[2] = px.col[2] & 0xf8; break;
		case FBF_IA88: mem[0] = mem[1] = mem[2] = px.col[0]; break;
		default: mem[0] = px.col[0]; mem[1] = px.col[1]; mem[2] = px.col[2]; break;
		}
		mem[3] = mc;
	}
	int mem_cov = mem[3] >> 5;
	bool blend_en, cvg_wrap, pass;
	int bshift[2];
	if (df & DB_DEPTH_TEST)
	{
		int memory_z = z_decompress(px.depth);
		int memory_dz = 1 << px.dz;
		int precision = (px.depth >> 11) & 0xf;
		bool coplanar = false;
		bshift[0] = clampi(int(sh.dz_compressed) - px.dz, 0, 4);
		bshift[1] = clampi(px.dz - int(sh.dz_compressed), 0, 4);
		if (precision < 3)
		{
			if (memory_dz != 0x8000) memory_dz = max(memory_dz << 1, 16 >> precision);
			else { coplanar = true; memory_dz = 0xffff; }
		}
		int cdz = int(sh.dz) | memory_dz;
		if (cdz != 0) cdz = 1 << find_msb(cdz);
		int cdz_i = cdz;
		cdz <<= 3;
		bool farther = coplanar || ((z + cdz) >= memory_z);
		bool overflow = (cov_count + mem_cov) >= 8;
		blend_en = force_blend || (!overflow && dba && farther);
		cvg_wrap = overflow;
		bool max_z = memory_z == 0x3ffff;
		bool front = z < memory_z;
		bool nearer = coplanar || ((z - cdz) <= memory_z);
		switch (sh.z_mode)
		{
		case 0: pass = max_z || (overflow ? front : nearer); break;
		case 1:
			if (!front || !farther || !overflow) pass = max_z || (overflow ? front : nearer);
			else
			{
				int e = max(find_msb(cdz_i & 0xffff), 0);
				int coeff = ((memory_z >> e) - (z >> e)) & 0xf;
				cov_count = min((coeff * cov_count) >> 3, 8);
				pass = true;
			}
			break;
		case 2: pass = front || max_z; break;
		default: pass = farther && nearer && !max_z; break;
		}
	}
	else
	{
		bshift[0] = 0;
		bshift[1] = min(0xf - int(sh.dz_compressed), 4);
		bool overflow = (cov_count + mem_cov) >= 8;
		blend_en = force_blend || (!overflow && dba);
		cvg_wrap = overflow;
		pass = true;
	}
	if (!(pass && (!dba || cov_count != 0))) return false;

	const bool color_on_cvg = (df & DB_COLOR_ON_CVG) != 0;
	int pixc[4] = { combined[0], combined[1], combined[2], combined[3] };
	const uint8_t *bm = sh.blend[0];
	if (df & DB_MULTI_CYCLE)
	{
		int tmp[3];
		blender(pixc, mem, sh.fog, sh.blend_color, shade_alpha, bm, force_blend, blend_en, color_on_cvg, cvg_wrap, bshift,
		        false, tmp);
		pixc[0] = tmp[0]; pixc[1] = tmp[1]; pixc[2] = tmp[2];
		bm = sh.blend[1];
	}
	int rgb[3];
	blender(pixc, mem, sh.fog, sh.blend_color, shade_alpha, bm, force_blend, blend_en, color_on_cvg, cvg_wrap, bshift,
	        true, rgb);
	if (df & DB_DITHER)
	{
		int dith = rgb_d;
#pragma unroll
		for (int c = 0; c < 3; c++)
		{
			int d = (dith >> (3 * c)) & 7;
			int o = rgb[c];
			int r = o > 247 ? 255 : ((o & 0xf8) + 8);
			int rs = (d - (o & 7)) >> 31;
			rgb[c] = (o + ((r - o) & rs)) & 0xff;
		}
	}
	int new_cov;
	switch (sh.coverage_mode)
	{
	case 0: new_cov = blend_en ? min(7, mem_cov + cov_count) : ((cov_count - 1) & 7); break;
	case 1: new_cov = (cov_count + mem_cov) & 7; break;
	case 2: new_cov = 7; break;
	default: new_cov = mem_cov; break;
	}
	write_color(ps.fb_fmt, px, rgb[0], rgb[1], rgb[2], (new_cov << 5) & 0xff);
	if (df & DB_DEPTH_UPDATE)
	{
		px.depth = z_compress(z);
		px.dz = sh.dz_compressed;
		px.ddirty = true;
		if (pc.alias) alias_d2c(ps.fb_fmt, px);
	}
	else if (pc.alias)
		alias_c2d(ps.fb_fmt, px);
	return true;
}


__device__ __forceinline__ bool shade_and_blend(const RdpPass &ps, const PassConst &pc, const RdpPrimGeom &g,
                                                const RdpPrimAttr &a, const RdpPrimShade &sh, const RdpTile *tiles,
                                                const uint16_t *tm, const SpanRow &sp, const SpanRow &sp_next, int x,
                                                int y, Pix &px)
{
	Shaded out;
	if (!shade_pixel(pc, g, a, sh, tiles, tm, sp, sp_next, x, y, out)) return false;
	return blend_pixel(ps, pc, sh, out, px);
}

// ============================================================================ pair list
// Exclusive scans of the per-tile pair counts (into pair offsets, the list of non-empty tiles
// and the launch's control words) and, for the primitive-major shading order, of the
// per-primitive pair counts (into each primitive's first position).  Counts are cleared for
// the next launch (the cleared per-primitive counts are k_expand's cursors).  Control words:
// [0] pairs, [1] 1 when the pairs or the span rows exceed the scratch capacity, [2] largest
// pair count seen, [3] non-empty tiles, [4] k_blend work counter (reset), [5] largest span-row
// count seen, [6..7] k_bin's 64-bit span-row counter (reset).

// One CTA of 1024 threads scans counts[0, num_items) in steps of 1024; `nonempty` optional.
// Leaves the total in *carry and the non-empty count in *carry_nz.
__device__ void cta_scan(uint32_t num_items, uint32_t *__restrict__ counts, uint32_t *__restrict__ offsets,
                         uint32_t *__restrict__ nonempty, uint32_t *warp_sums, uint32_t *warp_nz, uint32_t *carry,
                         uint32_t *carry_nz)
{
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	if (threadIdx.x == 0)
	{
		*carry = 0;
		*carry_nz = 0;
	}
	__syncthreads();
	for (uint32_t base = 0; base < num_items; base += 1024)
	{
		uint32_t i = base + threadIdx.x;
		uint32_t v = i < num_items ? counts[i] : 0u;
		if (i < num_items) counts[i] = 0u;
		uint32_t x = v;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1)
		{
			uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= o) x += y;
		}
		unsigned nzmask = __ballot_sync(0xffffffffu, v != 0);
		if (lane == 31)
		{
			warp_sums[wid] = x;
			warp_nz[wid] = __popc(nzmask);
		}
		__syncthreads();
		if (wid == 0)
		{
			uint32_t w = warp_sums[lane], z = warp_nz[lane];
#pragma unroll
			for (int o = 1; o < 32; o <<= 1)
			{
				uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
				uint32_t yz = __shfl_up_sync(0xffffffffu, z, o);
				if (lane >= o)
				{
					w += y;
					z += yz;
				}
			}
			warp_sums[lane] = w;
			warp_nz[lane] = z;
		}
		__syncthreads();
		uint32_t prefix = *carry + (wid ? warp_sums[wid - 1] : 0u) + x - v;
		uint32_t nz_pos = *carry_nz + (wid ? warp_nz[wid - 1] : 0u) + __popc(nzmask & ((1u << lane) - 1u));
		if (i < num_items) offsets[i] = prefix;
		if (v && nonempty) nonempty[nz_pos] = i;
		__syncthreads();
		if (threadIdx.x == 1023)
		{
			*carry = prefix + v;
			*carry_nz = nz_pos + (v ? 1u : 0u);
		}
		__syncthreads();
	}
}

// Writes the launch's control words from the pair total (one thread).  `capacity`: pairs (x)
// and span rows (y) the scratch holds; k_bin has counted the span rows in ctrl[6..7].
__device__ __forceinline__ void write_ctrl(uint32_t pairs, uint32_t nonempty_tiles, uint32_t *__restrict__ ctrl,
                                           uint2 capacity, uint32_t *__restrict__ pair_log, uint32_t log_slot)
{
	unsigned long long *row_counter = reinterpret_cast<unsigned long long *>(ctrl + 6);
	const unsigned long long rows = *row_counter;
	const bool over = pairs > capacity.x || rows > capacity.y;
	ctrl[0] = pairs;
	ctrl[1] = over ? 1u : 0u;
	ctrl[2] = max(ctrl[2], pairs); // largest pair count seen: the host grows the scratch to it
	ctrl[3] = nonempty_tiles;
	ctrl[4] = 0u;
	ctrl[5] = max(ctrl[5], uint32_t(min(rows, 0xffffffffull))); // largest span-row count seen
	*row_counter = 0ull;
	// Per-launch pair count for the autotuner; an overflowing launch is not a sample.
	if (pair_log) pair_log[log_slot] = over ? 0xffffffffu : pairs;
}

// Zeroes k_shade's work queues: the per-SM counters and their used-up bitmask.
__device__ __forceinline__ void clear_queues(uint32_t *__restrict__ queues, uint32_t num_queues)
{
	for (uint32_t q = threadIdx.x; q < num_queues + (num_queues + 31) / 32; q += blockDim.x) queues[q] = 0u;
}

// Single CTA: the tile scan, then (num_prims > 0) the primitive scan.
__global__ void __launch_bounds__(1024) k_scan(uint32_t num_items, uint32_t *__restrict__ counts,
                                               uint32_t *__restrict__ offsets, uint32_t *__restrict__ nonempty,
                                               uint32_t *__restrict__ ctrl, uint2 capacity,
                                               uint32_t *__restrict__ pair_log, uint32_t log_slot,
                                               uint32_t *__restrict__ queues, uint32_t num_queues, uint32_t num_prims,
                                               uint32_t *__restrict__ prim_counts, uint32_t *__restrict__ prim_offsets)
{
	__shared__ uint32_t warp_sums[32], warp_nz[32];
	__shared__ uint32_t carry, carry_nz;
	clear_queues(queues, num_queues);
	cta_scan(num_items, counts, offsets, nonempty, warp_sums, warp_nz, &carry, &carry_nz);
	if (threadIdx.x == 0)
	{
		offsets[num_items] = carry;
		write_ctrl(carry, carry_nz, ctrl, capacity, pair_log, log_slot);
	}
	__syncthreads();
	if (num_prims) cta_scan(num_prims, prim_counts, prim_offsets, nullptr, warp_sums, warp_nz, &carry, &carry_nz);
}

// Multi-CTA form for launches with many tiles or primitives: SCAN_TILE items per CTA.  The
// first `split` CTAs of k_scan_reduce / k_scan_down take the tiles, the rest the primitives.
// k_scan_reduce: per-CTA sums and non-empty counts; k_scan_top (1 CTA): their exclusive
// prefixes and the control words; k_scan_down: per-CTA scan plus prefix, offsets, tile list.
constexpr int SCAN_THREADS = 256, SCAN_PER_THREAD = 4, SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;

// Block-wide exclusive scan of one value per thread; returns the thread's prefix, *total the sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums, uint32_t *total)
{
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
	uint32_t x = v;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
		uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= o) x += y;
	}
	if (lane == 31) warp_sums[wid] = x;
	__syncthreads();
	if (wid == 0)
	{
		uint32_t w = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1)
		{
			uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
			if (lane >= o) w += y;
		}
		if (lane < nw) warp_sums[lane] = w;
	}
	__syncthreads();
	const uint32_t r = (wid ? warp_sums[wid - 1] : 0u) + x - v;
	*total = warp_sums[nw - 1];
	__syncthreads();
	return r;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(uint32_t num_items, const uint32_t *__restrict__ counts,
                                                             uint32_t *__restrict__ block_sums, uint32_t split,
                                                             uint32_t num_prims, const uint32_t *__restrict__ prim_counts,
                                                             uint32_t *__restrict__ prim_sums)
{
	__shared__ uint32_t warp_sums[32];
	uint32_t blk = blockIdx.x;
	if (blk >= split)
	{
		blk -= split;
		num_items = num_prims;
		counts = prim_counts;
		block_sums = prim_sums;
	}
	const uint32_t base = blk * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
	uint32_t sum = 0, nz = 0;
#pragma unroll
	for (int k = 0; k < SCAN_PER_THREAD; k++)
		if (base + k < num_items)
		{
			const uint32_t v = counts[base + k];
			sum += v;
			nz += v != 0;
		}
	uint32_t tot_sum, tot_nz;
	block_exclusive_scan(sum, warp_sums, &tot_sum);
	block_exclusive_scan(nz, warp_sums, &tot_nz);
	if (threadIdx.x == 0)
	{
		block_sums[2 * blk] = tot_sum;
		block_sums[2 * blk + 1] = tot_nz;
	}
}

// Exclusive prefixes of num_blocks (sum, non-empty) pairs in place; totals to *carry, *carry_nz.
__device__ void scan_block_sums(uint32_t num_blocks, uint32_t *__restrict__ block_sums, uint32_t *warp_sums,
                                uint32_t *carry, uint32_t *carry_nz)
{
	if (threadIdx.x == 0)
	{
		*carry = 0;
		*carry_nz = 0;
	}
	__syncthreads();
	for (uint32_t b0 = 0; b0 < num_blocks; b0 += 1024)
	{
		const uint32_t b = b0 + threadIdx.x;
		const uint32_t s = b < num_blocks ? block_sums[2 * b] : 0u, z = b < num_blocks ? block_sums[2 * b + 1] : 0u;
		uint32_t ts, tz;
		const uint32_t ps = block_exclusive_scan(s, warp_sums, &ts);
		const uint32_t pz = block_exclusive_scan(z, warp_sums, &tz);
		if (b < num_blocks)
		{
			block_sums[2 * b] = *carry + ps;
			block_sums[2 * b + 1] = *carry_nz + pz;
		}
		__syncthreads();
		if (threadIdx.x == 0)
		{
			*carry += ts;
			*carry_nz += tz;
		}
		__syncthreads();
	}
}

__global__ void __launch_bounds__(1024) k_scan_top(uint32_t num_blocks, uint32_t *__restrict__ block_sums,
                                                   uint32_t num_items, uint32_t *__restrict__ offsets,
                                                   uint32_t *__restrict__ ctrl, uint2 capacity,
                                                   uint32_t *__restrict__ pair_log, uint32_t log_slot,
                                                   uint32_t *__restrict__ queues, uint32_t num_queues,
                                                   uint32_t num_prim_blocks, uint32_t *__restrict__ prim_sums)
{
	__shared__ uint32_t warp_sums[32];
	__shared__ uint32_t carry, carry_nz;
	clear_queues(queues, num_queues);
	scan_block_sums(num_blocks, block_sums, warp_sums, &carry, &carry_nz);
	if (threadIdx.x == 0)
	{
		offsets[num_items] = carry;
		write_ctrl(carry, carry_nz, ctrl, capacity, pair_log, log_slot);
	}
	__syncthreads();
	if (num_prim_blocks) scan_block_sums(num_prim_blocks, prim_sums, warp_sums, &carry, &carry_nz);
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(uint32_t num_items, uint32_t *__restrict__ counts,
                                                           const uint32_t *__restrict__ block_sums,
                                                           uint32_t *__restrict__ offsets, uint32_t *__restrict__ nonempty,
                                                           uint32_t split, uint32_t num_prims,
                                                           uint32_t *__restrict__ prim_counts,
                                                           const uint32_t *__restrict__ prim_sums,
                                                           uint32_t *__restrict__ prim_offsets)
{
	__shared__ uint32_t warp_sums[32];
	uint32_t blk = blockIdx.x;
	if (blk >= split)
	{
		blk -= split;
		num_items = num_prims;
		counts = prim_counts;
		block_sums = prim_sums;
		offsets = prim_offsets;
		nonempty = nullptr;
	}
	const uint32_t base = blk * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
	uint32_t v[SCAN_PER_THREAD], sum = 0, nz = 0;
#pragma unroll
	for (int k = 0; k < SCAN_PER_THREAD; k++)
	{
		v[k] = base + k < num_items ? counts[base + k] : 0u;
		if (base + k < num_items) counts[base + k] = 0u;
		sum += v[k];
		nz += v[k] != 0;
	}
	uint32_t ts, tz;
	uint32_t ps = block_exclusive_scan(sum, warp_sums, &ts) + block_sums[2 * blk];
	uint32_t pz = block_exclusive_scan(nz, warp_sums, &tz) + block_sums[2 * blk + 1];
#pragma unroll
	for (int k = 0; k < SCAN_PER_THREAD; k++)
	{
		if (base + k < num_items)
		{
			offsets[base + k] = ps;
			if (v[k] && nonempty) nonempty[pz++] = base + k;
		}
		ps += v[k];
	}
}

// One warp per tile: turns the tile's primitive bitmask into its ordered run of
// (primitive, tile) pairs and clears the bitmask.
// With `featbits`, also writes the tile's scheduling features (sched.h) to features[item].
// With `list`, also places each pair in primitive-major order: list[prim_offsets[prim] + n] =
// {primitive, tx | ty << 16, pair index, pass}, n counted by prim_cursor (zeroed by k_scan_down);
// the order of one primitive's tiles is arbitrary, which changes no result.
// A warp step covers 128 bitmask words: each lane holds one 16-byte group and loads the next
// step's ahead.  The primitive-major slots (an atomic each) and the features are taken in a
// second loop over the tile's pairs just written, lanes in parallel, so no atomic waits in the
// bitmask walk.
__global__ void __launch_bounds__(256) k_expand(const RdpPass *__restrict__ passes, uint32_t num_passes, uint32_t num_items,
                         const uint32_t *__restrict__ offsets, const uint32_t *__restrict__ ctrl, uint2 *__restrict__ pairs,
                         const uint16_t *__restrict__ featbits, float *__restrict__ features, bool train,
                         const uint32_t *__restrict__ prim_offsets, uint32_t *__restrict__ prim_cursor,
                         uint4 *__restrict__ list)
{
	uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	int lane = threadIdx.x & 31;
	if (item >= num_items || ctrl[1]) return;
	const uint32_t pi = pass_of_item_warp(passes, num_passes, item, lane);
	const RdpPass &ps = passes[pi];
	uint32_t tl = item - ps.tile_item_begin;
	uint4 *masks = reinterpret_cast<uint4 *>(ps.masks + size_t(tl) * ps.mask_words);
	const uint32_t ngroups = (ps.prim_count + 127) / 128; // 16-byte groups holding bits
	const uint32_t first = offsets[item];
	const uint32_t npairs = offsets[item + 1] - first;
	if (!npairs) return;
	const uint32_t tile_xy = (tl % ps.tiles_x) | ((tl / ps.tiles_x) << 16); // tx | ty << 16
	const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
	uint32_t out = first;
	uint4 g = uint32_t(lane) < ngroups ? masks[lane] : zero;
	for (uint32_t base = 0; base < ngroups; base += 32)
	{
		const uint32_t gi = base + uint32_t(lane);
		const uint4 gn = gi + 32 < ngroups ? masks[gi + 32] : zero;
		const uint32_t c = __popc(g.x) + __popc(g.y) + __popc(g.z) + __popc(g.w);
		uint32_t x = c;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1)
		{
			uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= o) x += y;
		}
		uint32_t pos = out + x - c;
		out += __shfl_sync(0xffffffffu, x, 31);
		if (c)
		{
			masks[gi] = zero;
			for (int k = 0; k < 4; k++)
			{
				uint32_t wv = k == 0 ? g.x : k == 1 ? g.y : k == 2 ? g.z : g.w;
				while (wv)
				{
					const int b = __ffs(wv) - 1;
					wv &= wv - 1;
					pairs[pos++] = make_uint2(ps.prim_begin + (gi * 4 + uint32_t(k)) * 32 + uint32_t(b), item);
				}
			}
		}
		g = gn;
	}
	// Without training, only tiles the model evaluates need features.
	if (featbits && !train && npairs < RDP_SCHED_MIN_PAIRS) featbits = nullptr;
	if (!list && !featbits) return;
	__syncwarp(); // the lanes' pair entries are visible to the whole warp
	uint32_t fc[RDP_FEAT_COUNT];
#pragma unroll
	for (int i = 0; i < RDP_FEAT_COUNT; i++) fc[i] = 0;
	for (uint32_t p = first + uint32_t(lane); p < first + npairs; p += 32)
	{
		const uint32_t prim = pairs[p].x;
		if (list) list[prim_offsets[prim] + atomicAdd(&prim_cursor[prim], 1u)] = make_uint4(prim, tile_xy, p, pi);
		if (featbits)
		{
			const uint32_t fb = featbits[prim];
#pragma unroll
			for (int i = 0; i < RDP_FEAT_COUNT; i++) fc[i] += (fb >> i) & 1u;
		}
	}
	if (featbits)
	{
#pragma unroll
		for (int i = 0; i < RDP_FEAT_COUNT; i++)
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) fc[i] += __shfl_xor_sync(0xffffffffu, fc[i], o);
		if (lane < RDP_MLP_IN)
		{
			const float np = float(npairs), inv = 1.0f / np;
			float v;
			if (lane == 0) v = fminf(np, 1024.0f) * (1.0f / 64.0f);
			else if (lane == 1) v = log2f(1.0f + np) * 0.1f;
			else if (lane == 14)
				v = ps.fb_fmt == FBF_RGBA8888 ? 1.0f : (ps.fb_fmt == FBF_I8 || ps.fb_fmt == FBF_I4) ? 0.25f : 0.5f;
			else
			{
				const int f = lane == 15 ? RDP_FEAT_NOISE : lane - 2;
				uint32_t c = 0;
#pragma unroll
				for (int i = 0; i < RDP_FEAT_COUNT; i++)
					if (i == f) c = fc[i];
				v = float(c) * inv;
			}
			features[size_t(item) * RDP_MLP_IN + lane] = v;
		}
	}
}

// ============================================================================ k_shade
// Shading of every (tile, primitive) pair in parallel (the reference's rasterizer.comp): a few
// pairs per warp step (k_shade_packedn), the pixels that can be covered packed one per lane; two
// independent warps per CTA.  Results go to scratch as one
// 8-byte shaded record per pixel (pack_shaded).
constexpr int SHADE_THREADS = 64;

// Work distribution over positions (pairs).  Without queues, warp w of the grid shades
// positions w, w + warps, w + 2 warps, ...  With queues (one counter per SM, then a bitmask of
// used-up queues; zeroed by k_scan), positions are dealt in chunks of SHADE_CHUNK: queue q owns
// chunks q, q + nq, q + 2 nq, ..., and a warp takes positions from the queue of the SM it runs
// on (one atomic per position, issued a position ahead), so the warps of one SM shade
// neighbouring positions at the same time.  A warp that finds a queue used up marks it in the
// bitmask and moves to the next queue not marked; it exits only when every queue is marked, so
// every position is shaded whatever SMs the warps land on.  Launches with fewer than
// `queue_min` pairs per CTA use the fixed stride (the queues' first atomic and final sweep
// cost more than they gain there).  With `list` (k_expand), pair position j is the record
// list[j] = {primitive, tx | ty << 16, pair index, pass}: primitive-major order, so neighbouring
// positions mostly share a primitive (same shading path, state, spans and texels); without
// it, pair position j is pair j in tile order.  Lane 0 copies the next position's record into
// shared memory with cp.async while the warp shades the current one, so no global load chain
// sits between two positions.
constexpr uint32_t SHADE_CHUNK = 128;

// 16- or 8-byte asynchronous global -> shared copy (no registers held while in flight).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
	asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(uint32_t(__cvta_generic_to_shared(smem))),
	             "l"(gmem)
	             : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
	asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(uint32_t(__cvta_generic_to_shared(smem))),
	             "l"(gmem)
	             : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t sm_id()
{
	uint32_t r;
	asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
	return r;
}

__device__ __forceinline__ uint32_t queue_pos(uint32_t q, uint32_t k, uint32_t nq)
{
	return (q + (k / SHADE_CHUNK) * nq) * SHADE_CHUNK + k % SHADE_CHUNK;
}

// Next position after queue q was found used up; 0xffffffff once every queue is.  At most nq
// attempts: each failed one marks another queue.
__device__ __noinline__ uint32_t queue_steal(uint32_t *queues, uint32_t nq, uint32_t total, uint32_t &q)
{
	uint32_t *used = queues + nq;
	const uint32_t nw = (nq + 31) >> 5;
	atomicOr(&used[q >> 5], 1u << (q & 31));
	for (uint32_t attempt = 0; attempt < nq; attempt++)
	{
		const uint32_t start = q + 1 < nq ? q + 1 : 0u;
		uint32_t found = 0xffffffffu;
		for (uint32_t i = 0; i <= nw && found == 0xffffffffu; i++)
		{
			uint32_t w = (start >> 5) + i;
			w = w < nw ? w : w - nw;
			uint32_t open = ~*reinterpret_cast<volatile const uint32_t *>(used + w);
			if (w == nw - 1 && (nq & 31)) open &= (1u << (nq & 31)) - 1u;
			if (i == 0) open &= ~0u << (start & 31);
			if (open) found = w * 32 + uint32_t(__ffs(int(open)) - 1);
		}
		if (found == 0xffffffffu) return found;
		q = found;
		const uint32_t j = queue_pos(q, atomicAdd(&queues[q], 1u), nq);
		if (j < total) return j;
		atomicOr(&used[q >> 5], 1u << (q & 31));
	}
	return 0xffffffffu;
}

// Tile coordinates of a position's record: primitive-major records (k_expand) carry them packed
// as tx | ty << 16, tile-order pair entries carry the tile item.
__device__ __forceinline__ void record_tile(const RdpPass &ps, uint32_t y, bool packed, int &tx, int &ty)
{
	if (packed)
	{
		tx = int(y & 0xffffu);
		ty = int(y >> 16);
		return;
	}
	const uint32_t tl = y - ps.tile_item_begin;
	tx = int(tl % ps.tiles_x);
	ty = int(tl / ps.tiles_x);
}

// The shading kernels are compiled for several minimum residencies (register budgets); the
// executor's autotuner picks one.  More resident CTAs hide more latency at the price of some
// spilling.

// Packed shading: warps, no CTA barrier.  A warp takes NP positions per step (consecutive ones,
// so mostly tiles of one primitive in primitive-major order), picks the pairs' candidate pixels --
// inside the image and inside the valid span of their row (k_span's rows), the only ones that can
// be covered -- and shades just those, packed into as few 32-lane rounds as they fill: pairs with
// few covered pixels share rounds.  The other pixels are written as empty.  Per-pair data sits in
// shared memory for the shading rounds.  On the batched workload two pairs per step measured best
// (one pair 4 % slower, four slower than one: the rounds mix primitives).  SPEC selects the
// render-state variants of the shading code (shade_pixel_any).
template <int NP, int MIN_CTAS, bool SPEC>
__global__ void __launch_bounds__(SHADE_THREADS, MIN_CTAS)
	k_shade_packedn(const RdpPass *__restrict__ passes, uint32_t num_passes, const uint2 *__restrict__ pairs,
	                const uint32_t *__restrict__ ctrl, const RdpPrimGeom *__restrict__ geom,
	                const RdpPrimAttr *__restrict__ attr, const RdpPrimShade *__restrict__ shade,
	                const RdpTile *__restrict__ tilesets, uint2 *__restrict__ sc, const uint4 *__restrict__ list,
	                uint32_t *__restrict__ queues, uint32_t num_queues, uint32_t queue_min,
	                const SpanRow *__restrict__ spans, const uint32_t *__restrict__ prim_rows)
{
	static_assert(NP >= 2 && NP <= 4, "a candidate entry is slot << 6 | pixel in 8 bits");
	constexpr int WARPS = SHADE_THREADS / 32;
	constexpr uint32_t NONE = 0xffffffffu;
	struct Slot
	{
		uint32_t prim, pass, pr;
		int tx, ty, ylo;
		const SpanRow *rows;
	};
	__shared__ __align__(16) uint4 s_rec_all[WARPS][2][NP]; // [buffer][slot]: the positions' records
	__shared__ uint32_t s_pos_all[WARPS][2][NP];             // [buffer][slot]: positions (NONE: no pair)
	__shared__ Slot s_slot_all[WARPS][NP];
	__shared__ uint8_t s_px_all[WARPS][64 * NP];             // candidates: slot << 6 | pixel, in order
	if (ctrl[1]) return;
	const uint32_t total = ctrl[0];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	uint4(*s_rec)[NP] = s_rec_all[wid];
	uint32_t(*s_pos)[NP] = s_pos_all[wid];
	Slot *s_slot = s_slot_all[wid];
	uint8_t *s_px = s_px_all[wid];
	const uint32_t worker = blockIdx.x * WARPS + uint32_t(wid), workers = gridDim.x * WARPS;
	if (total < gridDim.x * queue_min) queues = nullptr;
	uint32_t q = 0, k_next = 0;
	int buf = 0;
	// Lane 0: the next step's positions into s_pos[b] and their records into s_rec[b].  With
	// queues a take reserves NP consecutive slots of the SM's queue; a take after stealing
	// reserves one.
	auto take = [&](int b, bool first) {
		uint32_t pos[NP];
#pragma unroll
		for (int i = 0; i < NP; i++) pos[i] = NONE;
		if (queues)
		{
			if (first)
			{
				q = sm_id() % num_queues;
				k_next = atomicAdd(&queues[q], uint32_t(NP));
			}
			uint32_t pa = queue_pos(q, k_next, num_queues);
			if (pa < total)
			{
				pos[0] = pa;
#pragma unroll
				for (int i = 1; i < NP; i++)
				{
					const uint32_t pi = queue_pos(q, k_next + uint32_t(i), num_queues);
					pos[i] = pi < total ? pi : NONE;
				}
			}
			else
			{
				pa = queue_steal(queues, num_queues, total, q);
				pos[0] = pa < total ? pa : NONE;
			}
			if (pa < total) k_next = atomicAdd(&queues[q], uint32_t(NP));
		}
		else
		{
			const uint32_t pa = first ? uint32_t(NP) * worker : s_pos[b ^ 1][0] + uint32_t(NP) * workers;
			if (pa < total)
#pragma unroll
				for (int i = 0; i < NP; i++) pos[i] = pa + uint32_t(i) < total ? pa + uint32_t(i) : NONE;
		}
#pragma unroll
		for (int i = 0; i < NP; i++)
		{
			if (pos[i] != NONE)
			{
				if (list) cp_async16(&s_rec[b][i], list + pos[i]);
				else cp_async8(&s_rec[b][i], pairs + pos[i]);
			}
			s_pos[b][i] = pos[i];
		}
	};
	if (lane == 0)
	{
		take(0, true);
		cp_async_wait_all();
	}
	__syncwarp();
	const unsigned below = (1u << lane) - 1u;
	while (s_pos[buf][0] != NONE)
	{
		__syncwarp();
		if (lane == 0) take(buf ^ 1, false);
		// Candidates of the pairs: pixels lane (rows 0-3) and lane + 32 (rows 4-7) of each.
		int count = 0;
#pragma unroll
		for (int s = 0; s < NP; s++)
		{
			const uint32_t pos = s_pos[buf][s];
			if (pos == NONE) break;
			const uint4 rec = s_rec[buf][s];
			const uint32_t prim = rec.x, pi = list ? rec.w : shade[prim].pass;
			const RdpPass &ps = passes[pi];
			int tx, ty;
			record_tile(ps, rec.y, list != nullptr, tx, ty);
			const RdpPrimGeom &g = geom[prim];
			const int fbw = int(ps.fb_width), fbh = int(ps.fb_height), ylo = g.span_ylo, yhi = g.span_yhi;
			const SpanRow *rows = spans + prim_rows[prim];
			const int x = tx * 8 + (lane & 7), y0 = ty * 8 + (lane >> 3), y1 = y0 + 4;
			bool c0 = x < fbw && y0 < fbh && y0 >= ylo && y0 <= yhi;
			bool c1 = x < fbw && y1 < fbh && y1 >= ylo && y1 <= yhi;
			if (c0)
			{
				const SpanRow &r = rows[y0 - ylo];
				c0 = r.valid && x >= r.start_x && x <= r.end_x;
			}
			if (c1)
			{
				const SpanRow &r = rows[y1 - ylo];
				c1 = r.valid && x >= r.start_x && x <= r.end_x;
			}
			const unsigned m0 = __ballot_sync(0xffffffffu, c0), m1 = __ballot_sync(0xffffffffu, c1);
			const int n0 = __popc(m0);
			if (c0) s_px[count + __popc(m0 & below)] = uint8_t((s << 6) | lane);
			if (c1) s_px[count + n0 + __popc(m1 & below)] = uint8_t((s << 6) | (lane + 32));
			count += n0 + __popc(m1);
			const uint32_t pr = list ? rec.z : pos;
			const size_t base = size_t(pr) * SHADE_THREADS;
			if (!c0) __stcs(sc + base + lane, kScratchEmpty);
			if (!c1) __stcs(sc + base + 32 + lane, kScratchEmpty);
			if (lane == 0) s_slot[s] = Slot{ prim, pi, pr, tx, ty, ylo, rows };
		}
		__syncwarp();
		for (int e = lane; e < count; e += 32)
		{
			const int ent = s_px[e], px = ent & 63;
			const Slot &sl = s_slot[ent >> 6];
			const RdpPass &ps = passes[sl.pass];
			PassConst pc;
			switch (ps.fb_fmt)
			{
			case FBF_I4: pc.fb_size = 0; pc.dx_mask = 0; pc.dx_shift = 0; break;
			case FBF_I8: pc.fb_size = 1; pc.dx_mask = ~7; pc.dx_shift = 3; break;
			case FBF_RGBA5551:
			case FBF_IA88: pc.fb_size = 2; pc.dx_mask = ~3; pc.dx_shift = 2; break;
			default: pc.fb_size = 4; pc.dx_mask = ~1; pc.dx_shift = 1; break;
			}
			pc.alias = ps.fb_addr == ps.depth_addr;
			const uint32_t prim = sl.prim;
			const RdpPrimShade &sh = shade[prim];
			const int y = sl.ty * 8 + (px >> 3);
			const SpanRow *sp = sl.rows + (y - sl.ylo);
			Shaded out;
			const bool ok = shade_pixel_any<SPEC>(pc, geom[prim], attr[prim], sh, tilesets + size_t(sh.tileset) * 8,
			                                      ps.tmem_snapshots + size_t(sh.tmem_index) * 2048, sp[0], sp[1],
			                                      sl.tx * 8 + (px & 7), y, out);
			__stcs(sc + size_t(sl.pr) * SHADE_THREADS + px, ok ? pack_shaded(out) : kScratchEmpty);
		}
		if (lane == 0) cp_async_wait_all();
		__syncwarp();
		buf ^= 1;
	}
}

// ============================================================================ k_blend
// One 64-thread CTA per tile: the tile's colour/depth stay in registers while its pairs are
// applied in primitive order (the reference's depth_blend.comp), then written back.
//
// The per-pair inputs come through shared memory: a ring of BLEND_STAGES stages, each holding up
// to BLEND_CHUNK consecutive pairs of the tile -- their shaded records (a tile's pairs are
// consecutive in the scratch, so one 1-D bulk copy moves them all) and each pair's primitive
// state (one 128-byte bulk copy per pair).  Thread 0 issues the copies up to BLEND_STAGES chunks
// ahead; they complete on the stage's mbarrier (transaction bytes).  So no global load sits in a
// pixel's serial chain of pairs.  Waits are bounded: a wait that gives up marks the CTA; at the
// chunk's barrier the CTA then sets bit 0 of the launch's error word (ctrl[8]), stops issuing,
// drains its own copies (bounded) and ends.
constexpr int BLEND_STAGES = 3, BLEND_CHUNK = 4;
constexpr uint32_t BLEND_WAIT_POLLS = 1u << 20; // mbarrier polls before a wait gives up
constexpr uint32_t BLEND_ERR_WAIT = 1u;

struct __align__(128) BlendStage
{
	uint2 rec[BLEND_CHUNK][SHADE_THREADS];     // shaded records, 512 bytes per pair
	RdpPrimShade shade[BLEND_CHUNK];           // primitive state, 128 bytes per pair
};
static_assert(sizeof(RdpPrimShade) == 128, "one bulk copy per primitive state");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
	uint32_t done;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(done)
	             : "r"(smem_u32(bar)), "r"(parity)
	             : "memory");
	return done != 0;
}
// Bounded wait for the phase with parity `parity` of `bar` to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
	for (uint32_t i = 0; i < BLEND_WAIT_POLLS; i++)
		if (mbar_try_wait(bar, parity)) return true;
	return false;
}
// 1-D bulk copy global -> shared completing on `bar` (16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smem_u32(dst)),
	             "l"(src), "r"(bytes), "r"(smem_u32(bar))
	             : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Thread 0: stage `st` receives pairs [first, first + count) of the scratch and their primitives'
// state; the copies complete on `bar`.
__device__ __forceinline__ void blend_issue(BlendStage &st, uint64_t *bar, uint32_t first, uint32_t count,
                                            const uint2 *__restrict__ pairs, const RdpPrimShade *__restrict__ shade,
                                            const uint2 *__restrict__ sc)
{
	fence_proxy_async_smem(); // the stage's previous contents were read through the generic proxy
	mbar_arrive_expect_tx(bar, count * (SHADE_THREADS * 8u + uint32_t(sizeof(RdpPrimShade))));
	bulk_g2s(&st.rec[0][0], sc + size_t(first) * SHADE_THREADS, count * SHADE_THREADS * 8u, bar);
	for (uint32_t k = 0; k < count; k++)
		bulk_g2s(&st.shade[k], shade + pairs[first + k].x, uint32_t(sizeof(RdpPrimShade)), bar);
}

// Returns false when a staging wait gave up (the error word is set; the CTA must stop).
__device__ __forceinline__ bool blend_tile(uint32_t item, const RdpPass *__restrict__ passes, uint32_t num_passes,
                                           const uint32_t *__restrict__ offsets, const uint2 *__restrict__ pairs,
                                           const RdpPrimShade *__restrict__ shade, const uint2 *__restrict__ sc,
                                           uint32_t *__restrict__ cycles, BlendStage *stages, uint64_t *bars,
                                           uint32_t &chunk_seq, uint32_t &issued_seq, uint32_t *__restrict__ err,
                                           volatile uint32_t *fail)
{
	const uint32_t p0 = offsets[item], p1 = offsets[item + 1];
	const int tid = threadIdx.x;
	if (p0 == p1)
	{
		if (cycles && tid == 0) cycles[item] = 0;
		return true;
	}
	const long long t_start = clock64();
	const uint32_t nchunks = (p1 - p0 + BLEND_CHUNK - 1) / BLEND_CHUNK;
	auto chunk_count = [&](uint32_t c) { return min(uint32_t(BLEND_CHUNK), p1 - p0 - c * BLEND_CHUNK); };
	// The first stages fill while the tile's pixels load.
	if (tid == 0)
		for (uint32_t c = 0; c < nchunks && c < uint32_t(BLEND_STAGES); c++)
		{
			const uint32_t sidx = (chunk_seq + c) % BLEND_STAGES;
			blend_issue(stages[sidx], &bars[sidx], p0 + c * BLEND_CHUNK, chunk_count(c), pairs, shade, sc);
			issued_seq++;
		}
	const uint32_t pi = pass_of_item_warp(passes, num_passes, item, int(threadIdx.x & 31));
	const RdpPass &ps = passes[pi];
	const uint32_t tl = item - ps.tile_item_begin;
	const int tx = int(tl % ps.tiles_x), ty = int(tl / ps.tiles_x);
	const int x = tx * 8 + (tid & 7), y = ty * 8 + (tid >> 3);
	const bool inside = x < int(ps.fb_width) && y < int(ps.fb_height);
	PassConst pc;
	switch (ps.fb_fmt)
	{
	case FBF_I4: pc.fb_size = 0; pc.dx_mask = 0; pc.dx_shift = 0; break;
	case FBF_I8: pc.fb_size = 1; pc.dx_mask = ~7; pc.dx_shift = 3; break;
	case FBF_RGBA5551:
	case FBF_IA88: pc.fb_size = 2; pc.dx_mask = ~3; pc.dx_shift = 2; break;
	default: pc.fb_size = 4; pc.dx_mask = ~1; pc.dx_shift = 1; break;
	}
	pc.alias = ps.fb_addr == ps.depth_addr;
	uint32_t addr_index;
	switch (ps.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8: addr_index = ps.fb_addr; break;
	case FBF_RGBA5551:
	case FBF_IA88: addr_index = ps.fb_addr >> 1; break;
	default: addr_index = ps.fb_addr >> 2; break;
	}
	const uint32_t ci = addr_index + ps.fb_width * uint32_t(y) + uint32_t(x);
	const uint32_t di = (ps.depth_addr >> 1) + ps.fb_width * uint32_t(y) + uint32_t(x);
	Pix px;
	uint32_t frags = 0;
	if (inside) load_pixel(ps, px, ci, di);
	for (uint32_t c = 0; c < nchunks; c++)
	{
		const uint32_t sidx = chunk_seq % BLEND_STAGES, parity = (chunk_seq / BLEND_STAGES) & 1u;
		if (!mbar_wait(&bars[sidx], parity)) *fail = 1u; // seen by all at the chunk's barrier
		const BlendStage &st = stages[sidx];
		const uint32_t cnt = chunk_count(c);
		if (inside)
			for (uint32_t k = 0; k < cnt; k++)
			{
				const uint2 rec = st.rec[k][tid];
				const uint32_t code = (rec.y >> 18) & 15u;
				if (code == SC_NONE) continue;
				const RdpPrimShade &sh = st.shade[k];
				Shaded in;
				in.combined = rec.x;
				in.shade_alpha = 0;
				if (code == SC_FILL)
				{
					in.coverage = 0x40;
					in.z_dith = 0;
				}
				else if (code == SC_COPY)
				{
					in.coverage = 0x20;
					in.z_dith = int(rec.y & 0xffffu);
				}
				else
				{
					in.coverage = int(code);
					in.shade_alpha = int(rec.y >> 22);
					const uint32_t noise = (sh.static_flags & RS_NEED_NOISE) ? reseed_noise(uint32_t(x), uint32_t(y), sh.prim_index) : 0u;
					in.z_dith = int((rec.y & 0x3ffffu) << 9) | rgb_dither_value(sh.static_flags, sh.dither, x, y, noise);
				}
				frags += blend_pixel(ps, pc, sh, in, px);
			}
		__syncthreads(); // every thread is done with the stage
		if (*fail)
		{
			if (tid == 0) atomicOr(err, BLEND_ERR_WAIT);
			return false;
		}
		if (tid == 0 && c + BLEND_STAGES < nchunks)
		{
			const uint32_t n = c + BLEND_STAGES;
			blend_issue(stages[sidx], &bars[sidx], p0 + n * BLEND_CHUNK, chunk_count(n), pairs, shade, sc);
			issued_seq++;
		}
		chunk_seq++;
	}
	if (inside) store_pixel(ps, px, ci, di, pc.alias);
	if (ps.wmask) mark_pixel(ps, px, ci, di, pc.alias, inside);
	unsigned long long *counters = ps.counters;
	if (counters)
	{
		unsigned long long total = frags;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
		if ((tid & 31) == 0 && total) atomicAdd(counters, total);
		if (tid == 0)
		{
			atomicAdd(counters + 1, 1ull);
			atomicAdd(counters + 2, (unsigned long long)(p1 - p0));
		}
	}
	if (cycles)
	{
		// Per-tile cost sample for the learned tile-order model: the slower warp's cycles.
		__syncthreads();
		if (tid == 0) cycles[item] = uint32_t(min(clock64() - t_start, 0xffffffffll));
	}
	return true;
}

// Persistent CTAs take non-empty tiles from a shared counter, in the order of `order`
// (longest predicted first) when given, else in tile order.  Each pixel's pairs form a serial
// dependency chain, so residency matters more than the few spills of a 40-register budget
// (24 CTAs per SM measured 8 % faster than 16 with 64 registers, 32 CTAs slower).
__global__ void __launch_bounds__(SHADE_THREADS, 24) k_blend(const RdpPass *__restrict__ passes, uint32_t num_passes,
                                                        const uint32_t *__restrict__ offsets,
                                                        const uint2 *__restrict__ pairs, uint32_t *__restrict__ ctrl,
                                                        const uint32_t *__restrict__ nonempty,
                                                        const RdpPrimShade *__restrict__ shade,
                                                        const uint2 *__restrict__ sc,
                                                        const uint32_t *__restrict__ order,
                                                        uint32_t *__restrict__ cycles)
{
	__shared__ BlendStage s_stage[BLEND_STAGES];
	__shared__ __align__(8) uint64_t s_bar[BLEND_STAGES];
	__shared__ uint32_t s_next, s_fail;
	if (ctrl[1]) return;
	if (threadIdx.x == 0)
	{
		s_fail = 0u;
		for (int i = 0; i < BLEND_STAGES; i++) mbar_init(&s_bar[i], 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
	const uint32_t n = ctrl[3];
	uint32_t chunk_seq = 0, issued_seq = 0; // chunks consumed / issued by this CTA (issued_seq: thread 0)
	for (;;)
	{
		if (threadIdx.x == 0) s_next = atomicAdd(&ctrl[4], 1u);
		__syncthreads();
		const uint32_t k = s_next;
		__syncthreads();
		if (k >= n) break;
		const uint32_t item = order ? order[k] : nonempty[k];
		if (!blend_tile(item, passes, num_passes, offsets, pairs, shade, sc, cycles, s_stage, s_bar, chunk_seq,
		                issued_seq, ctrl + 8, &s_fail))
		{
			// A wait gave up: the copies still in flight (issued, not consumed) finish before the
			// CTA's shared memory goes away, each wait bounded again.
			if (threadIdx.x == 0)
				for (uint32_t q = chunk_seq; q < issued_seq; q++)
					mbar_wait(&s_bar[q % BLEND_STAGES], (q / BLEND_STAGES) & 1u);
			break;
		}
	}
}

// ---------------------------------------------------------------------------- k_blend, register look-ahead
// The same blend with the per-pair inputs loaded straight from global memory: each thread keeps
// the shaded records and primitive indices of the next BLEND_AHEAD pairs in registers and
// prefetches their primitive state into L1.
__device__ __forceinline__ void blend_tile_lookahead(uint32_t item, const RdpPass *__restrict__ passes, uint32_t num_passes,
                                           const uint32_t *__restrict__ offsets, const uint2 *__restrict__ pairs,
                                           const RdpPrimShade *__restrict__ shade, const uint2 *__restrict__ sc,
                                           uint32_t *__restrict__ cycles)
{
	const uint32_t p0 = offsets[item], p1 = offsets[item + 1];
	if (p0 == p1)
	{
		if (cycles && threadIdx.x == 0) cycles[item] = 0;
		return;
	}
	const long long t_start = clock64();
	const uint32_t pi = pass_of_item_warp(passes, num_passes, item, int(threadIdx.x & 31));
	const RdpPass &ps = passes[pi];
	const uint32_t tl = item - ps.tile_item_begin;
	const int tx = int(tl % ps.tiles_x), ty = int(tl / ps.tiles_x);
	const int tid = threadIdx.x;
	const int x = tx * 8 + (tid & 7), y = ty * 8 + (tid >> 3);
	const bool inside = x < int(ps.fb_width) && y < int(ps.fb_height);
	PassConst pc;
	switch (ps.fb_fmt)
	{
	case FBF_I4: pc.fb_size = 0; pc.dx_mask = 0; pc.dx_shift = 0; break;
	case FBF_I8: pc.fb_size = 1; pc.dx_mask = ~7; pc.dx_shift = 3; break;
	case FBF_RGBA5551:
	case FBF_IA88: pc.fb_size = 2; pc.dx_mask = ~3; pc.dx_shift = 2; break;
	default: pc.fb_size = 4; pc.dx_mask = ~1; pc.dx_shift = 1; break;
	}
	pc.alias = ps.fb_addr == ps.depth_addr;
	uint32_t addr_index;
	switch (ps.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8: addr_index = ps.fb_addr; break;
	case FBF_RGBA5551:
	case FBF_IA88: addr_index = ps.fb_addr >> 1; break;
	default: addr_index = ps.fb_addr >> 2; break;
	}
	const uint32_t ci = addr_index + ps.fb_width * uint32_t(y) + uint32_t(x);
	const uint32_t di = (ps.depth_addr >> 1) + ps.fb_width * uint32_t(y) + uint32_t(x);
	Pix px;
	uint32_t frags = 0;
	if (inside)
	{
		load_pixel(ps, px, ci, di);
		// Software pipeline: the shaded record and primitive of pair pr + BLEND_AHEAD are loaded
		// (and its primitive's shading state prefetched into L1) while pair pr blends.
		constexpr int BLEND_AHEAD = 2;
		uint2 q_rec[BLEND_AHEAD];
		uint32_t q_prim[BLEND_AHEAD];
#pragma unroll
		for (int k = 0; k < BLEND_AHEAD; k++)
		{
			const uint32_t pr = p0 + uint32_t(k);
			q_rec[k] = kScratchEmpty;
			q_prim[k] = 0u;
			if (pr < p1)
			{
				q_rec[k] = __ldcs(sc + size_t(pr) * SHADE_THREADS + tid);
				q_prim[k] = pairs[pr].x;
				asm volatile("prefetch.global.L1 [%0];" ::"l"(shade + q_prim[k]));
			}
		}
		for (uint32_t pr = p0; pr < p1; pr++)
		{
			const uint2 rec = q_rec[0];
			const uint32_t prim = q_prim[0];
#pragma unroll
			for (int k = 0; k + 1 < BLEND_AHEAD; k++)
			{
				q_rec[k] = q_rec[k + 1];
				q_prim[k] = q_prim[k + 1];
			}
			const uint32_t nx = pr + BLEND_AHEAD;
			if (nx < p1)
			{
				q_rec[BLEND_AHEAD - 1] = __ldcs(sc + size_t(nx) * SHADE_THREADS + tid);
				q_prim[BLEND_AHEAD - 1] = pairs[nx].x;
				asm volatile("prefetch.global.L1 [%0];" ::"l"(shade + q_prim[BLEND_AHEAD - 1]));
			}
			const uint32_t code = (rec.y >> 18) & 15u;
			if (code == SC_NONE) continue;
			const RdpPrimShade &sh = shade[prim];
			Shaded in;
			in.combined = rec.x;
			in.shade_alpha = 0;
			if (code == SC_FILL)
			{
				in.coverage = 0x40;
				in.z_dith = 0;
			}
			else if (code == SC_COPY)
			{
				in.coverage = 0x20;
				in.z_dith = int(rec.y & 0xffffu);
			}
			else
			{
				in.coverage = int(code);
				in.shade_alpha = int(rec.y >> 22);
				const uint32_t noise = (sh.static_flags & RS_NEED_NOISE) ? reseed_noise(uint32_t(x), uint32_t(y), sh.prim_index) : 0u;
				in.z_dith = int((rec.y & 0x3ffffu) << 9) | rgb_dither_value(sh.static_flags, sh.dither, x, y, noise);
			}
			frags += blend_pixel(ps, pc, sh, in, px);
		}
		store_pixel(ps, px, ci, di, pc.alias);
	}
	if (ps.wmask) mark_pixel(ps, px, ci, di, pc.alias, inside);
	unsigned long long *counters = ps.counters;
	if (counters)
	{
		unsigned long long total = frags;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
		if ((tid & 31) == 0 && total) atomicAdd(counters, total);
		if (tid == 0)
		{
			atomicAdd(counters + 1, 1ull);
			atomicAdd(counters + 2, (unsigned long long)(p1 - p0));
		}
	}
	if (cycles)
	{
		// Per-tile cost sample for the learned tile-order model: the slower warp's cycles.
		__syncthreads();
		if (tid == 0) cycles[item] = uint32_t(min(clock64() - t_start, 0xffffffffll));
	}
}

// Persistent CTAs take non-empty tiles from a shared counter, in the order of `order`
// (longest predicted first) when given, else in tile order.  Each pixel's pairs form a serial
// dependency chain, so residency matters more than the few spills of a 40-register budget
// (24 CTAs per SM measured 8 % faster than 16 with 64 registers, 32 CTAs slower).
__global__ void __launch_bounds__(SHADE_THREADS, 24) k_blend_lookahead(const RdpPass *__restrict__ passes, uint32_t num_passes,
                                                        const uint32_t *__restrict__ offsets,
                                                        const uint2 *__restrict__ pairs, uint32_t *__restrict__ ctrl,
                                                        const uint32_t *__restrict__ nonempty,
                                                        const RdpPrimShade *__restrict__ shade,
                                                        const uint2 *__restrict__ sc,
                                                        const uint32_t *__restrict__ order,
                                                        uint32_t *__restrict__ cycles)
{
	__shared__ uint32_t s_next;
	if (ctrl[1]) return;
	const uint32_t n = ctrl[3];
	for (;;)
	{
		if (threadIdx.x == 0) s_next = atomicAdd(&ctrl[4], 1u);
		__syncthreads();
		const uint32_t k = s_next;
		__syncthreads();
		if (k >= n) break;
		const uint32_t item = order ? order[k] : nonempty[k];
		blend_tile_lookahead(item, passes, num_passes, offsets, pairs, shade, sc, cycles);
	}
}

// ============================================================================ k_raster
// One CTA of 64 threads per 8x8 tile, one pixel per thread; warp w owns rows 4w..4w+3.
// Both warps walk the tile's primitive bitmask in primitive order; pixel state stays in
// registers for the whole pass (init_tile/finish_tile, memory_interfacing.h:286-362).
constexpr int RASTER_THREADS = 64;

__device__ __forceinline__ void raster_tile(uint32_t item, const RdpPass *__restrict__ passes, uint32_t num_passes,
                                            const RdpPrimGeom *__restrict__ geom, const RdpPrimAttr *__restrict__ attr,
                                            const RdpPrimShade *__restrict__ shade, const RdpTile *__restrict__ tilesets)
{
	__shared__ SpanRow s_sp[2][5];
	__shared__ int s_any;
	const int wib = threadIdx.x >> 5;
	const int lane = threadIdx.x & 31;

	const uint32_t pi = pass_of_item_warp(passes, num_passes, item, int(threadIdx.x & 31));
	const RdpPass &ps = passes[pi];
	const uint32_t tile_linear = item - ps.tile_item_begin;
	const int tx = int(tile_linear % ps.tiles_x), ty = int(tile_linear / ps.tiles_x);
	uint32_t *masks = ps.masks + size_t(tile_linear) * ps.mask_words;
	const uint32_t nwords = (ps.prim_count + 31) / 32;

	PassConst pc;
	switch (ps.fb_fmt)
	{
	case FBF_I4: pc.fb_size = 0; pc.dx_mask = 0; pc.dx_shift = 0; break;
	case FBF_I8: pc.fb_size = 1; pc.dx_mask = ~7; pc.dx_shift = 3; break;
	case FBF_RGBA5551:
	case FBF_IA88: pc.fb_size = 2; pc.dx_mask = ~3; pc.dx_shift = 2; break;
	default: pc.fb_size = 4; pc.dx_mask = ~1; pc.dx_shift = 1; break;
	}
	pc.alias = ps.fb_addr == ps.depth_addr;
	uint32_t addr_index;
	switch (ps.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8: addr_index = ps.fb_addr; break;
	case FBF_RGBA5551:
	case FBF_IA88: addr_index = ps.fb_addr >> 1; break;
	default: addr_index = ps.fb_addr >> 2; break;
	}
	const uint32_t depth_index = ps.depth_addr >> 1;

	const int row0 = ty * 8 + wib * 4; // first row of this warp
	const int px_x = tx * 8 + (lane & 7);
	const int px_y = row0 + (lane >> 3);
	const int r = lane >> 3;
	const bool inside = px_x < int(ps.fb_width) && px_y < int(ps.fb_height);
	const uint32_t ci = addr_index + ps.fb_width * uint32_t(px_y) + uint32_t(px_x);
	const uint32_t di = depth_index + ps.fb_width * uint32_t(px_y) + uint32_t(px_x);

	Pix px;
	bool loaded = false;
	uint32_t frags = 0;

	for (uint32_t base = 0; base < nwords; base += 32)
	{
		uint32_t wi = base + lane;
		uint32_t wv = wi < nwords ? masks[wi] : 0u;
		unsigned nz = __ballot_sync(0xffffffffu, wv != 0);
		while (nz)
		{
			int src = __ffs(nz) - 1;
			nz &= nz - 1;
			uint32_t bits = __shfl_sync(0xffffffffu, wv, src);
			if (!loaded)
			{
				if (inside) load_pixel(ps, px, ci, di);
				loaded = true;
			}
			while (bits)
			{
				int b = __ffs(bits) - 1;
				bits &= bits - 1;
				uint32_t prim = ps.prim_begin + (base + src) * 32 + b;
				const RdpPrimGeom &g = geom[prim];
				const int ylo = g.span_ylo, yhi = g.span_yhi;
				if (yhi < row0 || ylo > row0 + 3) continue; // no row of this warp is covered
				// Spans for the warp's 4 rows plus the next row (pipelined texel1 peek).
				if (lane < 5)
					span_attr(g, attr[prim], row0 + lane, s_sp[wib][lane]);
				else if (lane >= 16 && lane < 21)
					span_x(g, row0 + (lane - 16), s_sp[wib][lane - 16]);
				__syncwarp();
				if (inside && px_y >= ylo && px_y <= yhi)
				{
					const RdpPrimShade &sh = shade[prim];
					frags += shade_and_blend(ps, pc, g, attr[prim], sh, tilesets + size_t(sh.tileset) * 8,
					                         ps.tmem_snapshots + size_t(sh.tmem_index) * 2048, s_sp[wib][r],
					                         s_sp[wib][r + 1], px_x, px_y, px);
				}
				__syncwarp();
			}
		}
	}
	if (loaded && inside) store_pixel(ps, px, ci, di, pc.alias);
	if (ps.wmask) mark_pixel(ps, px, ci, di, pc.alias, loaded && inside);

	// Both warps have consumed the bitmask: clear it for the next pass using this slot.
	if (threadIdx.x == 0) s_any = 0;
	__syncthreads();
	if (loaded && lane == 0) s_any = 1;
	__syncthreads();
	unsigned long long pairs_here = 0;
	if (s_any)
		for (uint32_t wi = threadIdx.x; wi < nwords; wi += RASTER_THREADS)
		{
			pairs_here += __popc(masks[wi]);
			masks[wi] = 0u;
		}

	unsigned long long *fragments = ps.counters;
	if (fragments)
	{
		unsigned long long total = frags;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1)
		{
			total += __shfl_xor_sync(0xffffffffu, total, o);
			pairs_here += __shfl_xor_sync(0xffffffffu, pairs_here, o);
		}
		if (lane == 0 && total) atomicAdd(fragments, total);
		if (lane == 0 && pairs_here) atomicAdd(fragments + 2, pairs_here);
		if (threadIdx.x == 0 && s_any) atomicAdd(fragments + 1, 1ull);
	}
}

// Fallback when the pair list overflowed the scratch capacity (ctrl[1]): persistent CTAs,
// each shading and blending whole tiles; without overflow every CTA returns at once.
__global__ void __launch_bounds__(RASTER_THREADS) k_raster(const RdpPass *__restrict__ passes, uint32_t num_passes,
                                                          uint32_t num_items, const RdpPrimGeom *__restrict__ geom,
                                                          const RdpPrimAttr *__restrict__ attr,
                                                          const RdpPrimShade *__restrict__ shade,
                                                          const RdpTile *__restrict__ tilesets,
                                                          const uint32_t *__restrict__ ctrl)
{
	if (!ctrl[1]) return;
	for (uint32_t item = blockIdx.x; item < num_items; item += gridDim.x)
	{
		raster_tile(item, passes, num_passes, geom, attr, shade, tilesets);
		__syncthreads();
	}
}

// ============================================================================ k_fill
// Launches whose primitives all take the fill pipe (cycle type 3: a frame's clears;
// RdpLaunch.fill_only).  A pixel takes the fill colour wherever x lies in its row's span
// (shading.h:55-62 with the fill branch of memory_interfacing.h:381-571), so only the x extent of
// each row is set up and no shading record is built.  One warp per 8x8 tile, independent of the
// CTA's other warps: lane l owns pixels (l % 8, l / 8) and (l % 8, l / 8 + 4) of the tile, and the
// warp alone clears the bitmask words it consumed.
constexpr int FILL_THREADS = 256, FILL_TILES = 4; // tiles per warp, consecutive items

// Marks the colour bytes of a fill's stored pixels (px.cdirty) in the write mask.  The 8 pixels
// of a tile row (lanes 8r .. 8r+7) hold at most 32 contiguous bytes -- at most two mask words,
// also where the address wraps -- so each row's lanes merge their bits with three reductions and
// one lane issues at most two atomics.
__device__ __forceinline__ void mark_fill_row(const RdpPass &p, const Pix &px, uint32_t ci, int lane)
{
	uint32_t ca, cn;
	switch (p.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8: ca = (ci & (p.rdram_size - 1)) ^ 3u; cn = 1; break;
	case FBF_RGBA5551:
	case FBF_IA88: ca = ((ci & ((p.rdram_size >> 1) - 1)) ^ 1u) * 2u; cn = 2; break;
	default: ca = (ci & ((p.rdram_size >> 2) - 1)) * 4u; cn = 4; break;
	}
	const bool c = px.cdirty;
	const uint32_t word = ca >> 5, bits = c ? ((1u << cn) - 1u) << (ca & 31u) : 0u;
	const unsigned row = 0xffu << (lane & 24);
	const uint32_t lo = __reduce_min_sync(row, c ? word : 0xffffffffu);
	const uint32_t hi = __reduce_max_sync(row, c ? word : 0u);
	const uint32_t blo = __reduce_or_sync(row, word == lo ? bits : 0u);
	const uint32_t bhi = __reduce_or_sync(row, word != lo ? bits : 0u);
	if ((lane & 7) == 0)
	{
		if (blo) atomicOr(p.wmask + lo, blo);
		if (bhi) atomicOr(p.wmask + hi, bhi);
	}
}

// One 8x8 tile of a fill-only launch (k_fill).  Returns whether any primitive was binned there;
// adds the fragments and binned primitives to frags / pairs.
// The x extents in s_sp belong to primitive *sp_prim at tile row *sp_row0 (shared by the tiles of
// one row of the image, so consecutive tiles reuse them).
__device__ __forceinline__ bool fill_tile(const RdpPass &ps, uint32_t tile_linear, int tx, int ty,
                                          const RdpPrimGeom *__restrict__ geom,
                                          const RdpPrimShade *__restrict__ shade, SpanRow *s_sp, uint32_t &sp_prim,
                                          int &sp_row0, int lane, uint32_t &frags, uint32_t &pairs)
{
	uint32_t *masks = ps.masks + size_t(tile_linear) * ps.mask_words;
	const uint32_t nwords = (ps.prim_count + 31) / 32;

	PassConst pc;
	pc.fb_size = pc.dx_mask = pc.dx_shift = 0; // the fill pipe reads neither
	pc.alias = ps.fb_addr == ps.depth_addr;
	uint32_t addr_index;
	switch (ps.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8: addr_index = ps.fb_addr; break;
	case FBF_RGBA5551:
	case FBF_IA88: addr_index = ps.fb_addr >> 1; break;
	default: addr_index = ps.fb_addr >> 2; break;
	}
	const uint32_t depth_index = ps.depth_addr >> 1;

	const int row0 = ty * 8;
	const int px_x = tx * 8 + (lane & 7);
	const int y0 = row0 + (lane >> 3), y1 = y0 + 4;
	const bool in0 = px_x < int(ps.fb_width) && y0 < int(ps.fb_height);
	const bool in1 = px_x < int(ps.fb_width) && y1 < int(ps.fb_height);
	const uint32_t ci0 = addr_index + ps.fb_width * uint32_t(y0) + uint32_t(px_x);
	const uint32_t di0 = depth_index + ps.fb_width * uint32_t(y0) + uint32_t(px_x);
	const uint32_t ci1 = ci0 + 4u * ps.fb_width, di1 = di0 + 4u * ps.fb_width;

	// The fill pipe sets every stored field of a pixel from the fill colour alone (colour, coverage
	// bits, the aliased depth; never the depth image) and a pixel no fill covers is not stored, so
	// nothing is loaded.
	Pix p0, p1;
	p0.cidx = ci0;
	p1.cidx = ci1;
	p0.cdirty = p0.ddirty = p1.cdirty = p1.ddirty = false;
	p0.depth = p0.dz = p1.depth = p1.dz = 0;
#pragma unroll
	for (int c = 0; c < 4; c++) p0.col[c] = p1.col[c] = 0;
	bool any = false;
	for (uint32_t base = 0; base < nwords; base += 32)
	{
		const uint32_t wi = base + lane;
		const uint32_t wv = wi < nwords ? masks[wi] : 0u;
		unsigned nz = __ballot_sync(0xffffffffu, wv != 0);
		any = any || nz != 0;
		while (nz)
		{
			const int src = __ffs(nz) - 1;
			nz &= nz - 1;
			uint32_t bits = __shfl_sync(0xffffffffu, wv, src);
			while (bits)
			{
				const int b = __ffs(bits) - 1;
				bits &= bits - 1;
				const uint32_t prim = ps.prim_begin + (base + src) * 32 + b;
				const RdpPrimGeom &g = geom[prim];
				const uint32_t col = shade[prim].fill_color;
				const int ylo = g.span_ylo, yhi = g.span_yhi;
				if (yhi < row0 || ylo > row0 + 7) continue; // no row of the tile is covered
				if (prim != sp_prim || row0 != sp_row0)
				{
					__syncwarp();
					if (lane < 8) span_x(g, row0 + lane, s_sp[lane]);
					sp_prim = prim;
					sp_row0 = row0;
					__syncwarp();
				}
				const SpanRow &a = s_sp[lane >> 3], &c = s_sp[(lane >> 3) + 4];
				if (in0 && y0 >= ylo && y0 <= yhi && a.valid && px_x >= a.start_x && px_x <= a.end_x)
					frags += fill_pixel(ps, pc, col, p0);
				if (in1 && y1 >= ylo && y1 <= yhi && c.valid && px_x >= c.start_x && px_x <= c.end_x)
					frags += fill_pixel(ps, pc, col, p1);
			}
		}
	}
	if (!any) return false; // no primitive binned here: nothing stored, marked or counted
	if (in0) store_pixel(ps, p0, ci0, di0, pc.alias);
	if (in1) store_pixel(ps, p1, ci1, di1, pc.alias);
	if (ps.wmask)
	{
		mark_fill_row(ps, p0, ci0, lane);
		mark_fill_row(ps, p1, ci1, lane);
	}
	// The warp has consumed the bitmask: clear it for the next pass using this slot.
	for (uint32_t wi = lane; wi < nwords; wi += 32)
	{
		pairs += __popc(masks[wi]);
		masks[wi] = 0u;
	}
	return true;
}

// One warp per FILL_TILES consecutive tiles (mostly of one pass: the pass is looked up again only
// when a tile leaves the current one), independent of the CTA's other warps: lane l owns pixels
// (l % 8, l / 8) and (l % 8, l / 8 + 4) of each tile, and the warp alone clears the bitmask
// words it consumed.  A pass's counters take one update per warp.
__global__ void __launch_bounds__(FILL_THREADS, 4) k_fill(const RdpPass *__restrict__ passes, uint32_t num_passes,
                                                      uint32_t num_items, const RdpPrimGeom *__restrict__ geom,
                                                      const RdpPrimShade *__restrict__ shade)
{
	__shared__ SpanRow s_sp[FILL_THREADS / 32][8];
	const int wib = threadIdx.x >> 5;
	const int lane = threadIdx.x & 31;
	const uint32_t first = (blockIdx.x * (FILL_THREADS / 32) + uint32_t(wib)) * FILL_TILES;
	uint32_t pi = 0, begin = 1, end = 0; // the current pass and its tile items [begin, end)
	uint32_t frags = 0, pairs = 0, tiles = 0;
	int tx = 0, ty = 0; // of the next tile of the current pass
	uint32_t sp_prim = 0xffffffffu;
	int sp_row0 = -1;
	auto flush = [&]() {
		unsigned long long *counters = passes[pi].counters;
		if (!counters || !tiles) return;
		unsigned long long f = frags, pr = pairs;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1)
		{
			f += __shfl_xor_sync(0xffffffffu, f, o);
			pr += __shfl_xor_sync(0xffffffffu, pr, o);
		}
		if (lane == 0)
		{
			if (f) atomicAdd(counters, f);
			atomicAdd(counters + 1, (unsigned long long)tiles);
			atomicAdd(counters + 2, pr);
		}
	};
	for (uint32_t k = 0; k < uint32_t(FILL_TILES); k++)
	{
		const uint32_t item = first + k;
		if (item >= num_items) break; // the whole warp
		if (item < begin || item >= end)
		{
			if (begin < end) flush();
			frags = pairs = tiles = 0;
			pi = pass_of_item_warp(passes, num_passes, item, lane);
			begin = passes[pi].tile_item_begin;
			end = begin + passes[pi].tiles_x * passes[pi].tiles_y;
			tx = int((item - begin) % passes[pi].tiles_x);
			ty = int((item - begin) / passes[pi].tiles_x);
			sp_prim = 0xffffffffu; // primitive indices are per launch, so a new pass keeps none
		}
		if (fill_tile(passes[pi], item - begin, tx, ty, geom, shade, s_sp[wib], sp_prim, sp_row0, lane, frags,
		              pairs))
			tiles++;
		if (++tx == int(passes[pi].tiles_x))
		{
			tx = 0;
			ty++;
		}
	}
	if (begin < end) flush();
}

// ============================================================================ k_raster_upscaled
// The upscaled pass (depth_blend.comp with SCALING_LOG2 > 0, rdp_renderer.cpp:2287-2342): one 8x8
// tile of the scaled image per CTA, its binned primitives walked in order, shading and blending
// fused as in k_raster.  Scanline y of the scaled image has its own span row (span_setup.comp
// with the factor), computed per primitive for the warp's rows.  Pixel (x, y) reads and writes
// sample slice (y % S) * S + x % S of the multisampled RDRAM at native pixel (x / S, y / S)
// (memory_interfacing.h:286-362).  Primitives drawn at native resolution
// (TRIANGLE_SETUP_DISABLE_UPSCALING_BIT) shade every pixel at the top-left sample of its native
// pixel (shading.h:45-52).  With super-sampled readback each written pixel sets its native
// pixel's colour / depth bits in the write mask (emit_scaled_write_masks, memory_interfacing.h:
// 305-337), which the resolve reads.
__device__ __forceinline__ void raster_tile_upscaled(uint32_t item, const RdpPass *__restrict__ passes,
                                                     uint32_t num_passes, const RdpPrimGeom *__restrict__ geom,
                                                     const RdpPrimAttr *__restrict__ attr,
                                                     const RdpPrimShade *__restrict__ shade,
                                                     const RdpTile *__restrict__ tilesets)
{
	__shared__ SpanRow s_sp[2][5];
	const int wib = threadIdx.x >> 5;
	const int lane = threadIdx.x & 31;

	const uint32_t pi = pass_of_item_warp(passes, num_passes, item, int(threadIdx.x & 31));
	const RdpPass &ps = passes[pi];
	const uint32_t tile_linear = item - ps.tile_item_begin;
	const int tx = int(tile_linear % ps.tiles_x), ty = int(tile_linear / ps.tiles_x);
	uint32_t *masks = ps.masks + size_t(tile_linear) * ps.mask_words;
	const uint32_t nwords = (ps.prim_count + 31) / 32;
	const int sl = int(ps.scale & 3u), S = 1 << sl;

	PassConst pc;
	switch (ps.fb_fmt)
	{
	case FBF_I4: pc.fb_size = 0; pc.dx_mask = 0; pc.dx_shift = 0; break;
	case FBF_I8: pc.fb_size = 1; pc.dx_mask = ~7; pc.dx_shift = 3; break;
	case FBF_RGBA5551:
	case FBF_IA88: pc.fb_size = 2; pc.dx_mask = ~3; pc.dx_shift = 2; break;
	default: pc.fb_size = 4; pc.dx_mask = ~1; pc.dx_shift = 1; break;
	}
	pc.alias = ps.fb_addr == ps.depth_addr;
	pc.sl = sl;
	uint32_t addr_index;
	switch (ps.fb_fmt)
	{
	case FBF_I4:
	case FBF_I8: addr_index = ps.fb_addr; break;
	case FBF_RGBA5551:
	case FBF_IA88: addr_index = ps.fb_addr >> 1; break;
	default: addr_index = ps.fb_addr >> 2; break;
	}
	const uint32_t depth_index = ps.depth_addr >> 1;

	const int row0 = ty * 8 + wib * 4;
	const int px_x = tx * 8 + (lane & 7);
	const int px_y = row0 + (lane >> 3);
	const bool inside = px_x < int(ps.fb_width) && px_y < int(ps.fb_height);
	const uint32_t native_w = ps.fb_width >> sl;
	const uint32_t xn = uint32_t(px_x) >> sl, yn = uint32_t(px_y) >> sl;
	const uint32_t slice = ((uint32_t(px_y) & uint32_t(S - 1)) << sl) + (uint32_t(px_x) & uint32_t(S - 1));
	const uint32_t ci = addr_index + native_w * yn + xn;
	const uint32_t di = depth_index + native_w * yn + xn;
	// This pixel's sample slice of the multisampled copies.
	RdpPass sp = ps;
	sp.rdram = ps.rdram + size_t(slice) * ps.rdram_size;
	sp.hidden = ps.hidden + size_t(slice) * (ps.rdram_size >> 1);
	sp.wmask = nullptr;

	Pix px;
	bool loaded = false;
	for (uint32_t base = 0; base < nwords; base += 32)
	{
		uint32_t wi = base + lane;
		uint32_t wv = wi < nwords ? masks[wi] : 0u;
		unsigned nz = __ballot_sync(0xffffffffu, wv != 0);
		while (nz)
		{
			int src = __ffs(nz) - 1;
			nz &= nz - 1;
			uint32_t bits = __shfl_sync(0xffffffffu, wv, src);
			if (!loaded)
			{
				if (inside) load_pixel(sp, px, ci, di);
				loaded = true;
			}
			while (bits)
			{
				int b = __ffs(bits) - 1;
				bits &= bits - 1;
				uint32_t prim = ps.prim_begin + (base + src) * 32 + b;
				const RdpPrimGeom &g = geom[prim];
				const int ylo = g.span_ylo << sl, yhi = (g.span_yhi << sl) + S - 1;
				if (yhi < row0 || ylo > row0 + 3) continue; // no row of this warp is covered
				const bool native_res = (g.flags & TRI_DISABLE_UPSCALING) != 0;
				// Rows rb .. rb + 4 hold every (masked) row of the warp and the next row.
				const int rb = native_res ? (row0 & ~(S - 1)) : row0;
				if (lane < 5)
					span_attr(g, attr[prim], rb + lane, s_sp[wib][lane], sl);
				else if (lane >= 16 && lane < 21)
					span_x(g, rb + (lane - 16), s_sp[wib][lane - 16], sl);
				__syncwarp();
				if (inside && px_y >= ylo && px_y <= yhi)
				{
					const int xs = native_res ? (px_x & ~(S - 1)) : px_x;
					const int ys = native_res ? (px_y & ~(S - 1)) : px_y;
					const RdpPrimShade &sh = shade[prim];
					shade_and_blend(ps, pc, g, attr[prim], sh, tilesets + size_t(sh.tileset) * 8,
					                ps.tmem_snapshots + size_t(sh.tmem_index) * 2048, s_sp[wib][ys - rb],
					                s_sp[wib][ys - rb + 1], xs, ys, px);
				}
				__syncwarp();
			}
		}
	}
	if (loaded && inside)
	{
		store_pixel(sp, px, ci, di, pc.alias);
		if (ps.scale & 0x100u)
		{
			const uint32_t word = (uint32_t(px.cdirty) + 2u * uint32_t(px.ddirty)) << (2 * ((xn & 3) + (yn & 3) * 4));
			uint32_t *wm = reinterpret_cast<uint32_t *>(ps.rdram + (size_t(ps.rdram_size) << (2 * sl)));
			if (word) atomicOr(wm + (yn >> 2) * ((native_w + 3) >> 2) + (xn >> 2), word);
		}
	}
	// Clear the bitmask words this tile consumed for the next pass using the slot.
	__syncthreads();
	for (uint32_t wi = threadIdx.x; wi < nwords; wi += RASTER_THREADS) masks[wi] = 0u;
}

__global__ void __launch_bounds__(RASTER_THREADS) k_raster_upscaled(const RdpPass *__restrict__ passes,
                                                                   uint32_t num_passes, uint32_t num_items,
                                                                   const RdpPrimGeom *__restrict__ geom,
                                                                   const RdpPrimAttr *__restrict__ attr,
                                                                   const RdpPrimShade *__restrict__ shade,
                                                                   const RdpTile *__restrict__ tilesets)
{
	for (uint32_t item = blockIdx.x; item < num_items; item += gridDim.x)
	{
		raster_tile_upscaled(item, passes, num_passes, geom, attr, shade, tilesets);
		__syncthreads();
	}
}

} // namespace rdp

// ============================================================================ host launchers
extern "C" cudaError_t rdp_kernels_init_luts(const uint8_t *blender_lut)
{
	return cudaMemcpyToSymbol(rdp::g_blender_lut, blender_lut, 0x8000);
}

namespace {
typedef void (*ShadeKernel)(const RdpPass *, uint32_t, const uint2 *, const uint32_t *, const RdpPrimGeom *,
                            const RdpPrimAttr *, const RdpPrimShade *, const RdpTile *, uint2 *, const uint4 *,
                            uint32_t *, uint32_t, uint32_t, const rdp::SpanRow *, const uint32_t *);
const ShadeKernel kShadeVariants[RDP_SHADE_VARIANTS] = {
	rdp::k_shade_packedn<2, 18, false>, rdp::k_shade_packedn<3, 16, false>, rdp::k_shade_packedn<4, 16, false>,
	rdp::k_shade_packedn<4, 18, false>, rdp::k_shade_packedn<2, 16, true>,  rdp::k_shade_packedn<2, 18, true>,
	rdp::k_shade_packedn<2, 20, true>,  rdp::k_shade_packedn<2, 24, true>
};
} // namespace

extern "C" int rdp_kernels_blend_ctas_per_sm(int kernel)
{
	int n = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel ? rdp::k_blend : rdp::k_blend_lookahead,
	                                                  rdp::SHADE_THREADS, 0) != cudaSuccess)
		n = 8;
	return n > 0 ? n : 1;
}

extern "C" int rdp_kernels_shade_ctas_per_sm(int variant)
{
	if (variant < 0 || variant >= RDP_SHADE_VARIANTS) variant = 0;
	int n = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kShadeVariants[variant], rdp::SHADE_THREADS, 0) !=
	    cudaSuccess)
		n = 8;
	return n > 0 ? n : 1;
}

// Launches with many tiles (or, in primitive-major order, many primitives) scan with several CTAs.
static bool multi_cta_scan(const RdpLaunch *L)
{
	return L->scan_blocks && (L->num_tile_items > RDP_SCAN_SINGLE_CTA_MAX ||
	                          (L->shade_list && L->prim_scan_blocks && L->num_prims > RDP_SCAN_SINGLE_CTA_MAX));
}

// Warps that share each warp's (primitive, tile) tests in k_bin (its grid's y dimension) when no
// per-primitive count is taken: a launch of few primitives still fills the GPU.
static uint32_t bin_split(const RdpLaunch *L)
{
	const uint32_t target = std::max<uint32_t>(L->num_sms, 1u) * 32u;
	const uint32_t warps = std::max<uint32_t>((L->num_prims + 31) / 32, 1u);
	return std::min<uint32_t>(std::max<uint32_t>(target / warps, 1u), 1024u);
}

extern "C" uint32_t rdp_kernels_count(const RdpLaunch *L)
{
	uint32_t n = 0;
	if (L->upscaled || L->fill_only)
		return (L->num_prims ? 2u : 0u) + (L->num_tmem_passes ? 2u : 0u) + (L->num_prims && L->num_tile_items ? 1u : 0u);
	if (L->num_prims) n += 2;
	if (L->num_prims && L->num_tile_items && L->spans) n += 1;
	if (L->num_tmem_passes) n += 2;
	if (L->num_prims && L->num_tile_items)
	{
		n += 5;
		if (multi_cta_scan(L)) n += 2;
		if (L->sched && (L->sched->order_enabled || L->sched->train_enabled))
		{
			n += 3;
			if (L->sched->train_enabled && L->tile_cycles) n += 3;
		}
	}
	return n;
}

extern "C" cudaError_t rdp_kernels_launch(const RdpLaunch *L, cudaStream_t stream)
{
	if (L->upscaled)
	{
		// Upscaled passes: set-up, binning at the scaled resolution, TMEM (super-sampled readback
		// applies the pass's uploads here) and the fused per-tile kernel.
		if (L->num_prims)
		{
			rdp::k_prim_setup<<<(L->num_prims + 127) / 128, 128, 0, stream>>>(L->prims_in, L->num_prims, L->words,
			                                                                   L->state_blocks, L->passes,
			                                                                   L->num_passes, L->geom, L->attr,
			                                                                   L->shade, nullptr);
			rdp::k_bin<<<dim3((L->num_prims + 255) / 256, bin_split(L)), 256, 0, stream>>>(
				L->num_prims, L->geom, L->shade, L->passes, nullptr, nullptr);
		}
		if (L->num_tmem_passes)
		{
			rdp::k_tmem_apply<<<L->num_uploads, 256, 0, stream>>>(L->passes, L->tmem_pass_list, L->num_tmem_passes,
			                                                      L->uploads, L->tmem_keep);
			rdp::k_tmem_carry<<<dim3(2048 / 32, L->num_tmem_passes), rdp::TMEM_CARRY_WARPS * 32, 0, stream>>>(
				L->passes, L->tmem_carry_list, L->tmem_keep);
		}
		if (L->num_prims && L->num_tile_items)
			rdp::k_raster_upscaled<<<std::min<uint32_t>(L->num_tile_items, L->blend_ctas), rdp::RASTER_THREADS, 0,
			                         stream>>>(L->passes, L->num_passes, L->num_tile_items, L->geom, L->attr,
			                                   L->shade, L->tilesets);
		return cudaGetLastError();
	}
	if (L->fill_only)
	{
		// Fill-only passes: set-up, binning, TMEM, and one per-tile kernel (no pair list).
		if (L->num_prims)
		{
			rdp::k_prim_setup<<<(L->num_prims + 127) / 128, 128, 0, stream>>>(L->prims_in, L->num_prims, L->words,
			                                                                   L->state_blocks, L->passes,
			                                                                   L->num_passes, L->geom, L->attr,
			                                                                   L->shade, nullptr);
			rdp::k_bin<<<dim3((L->num_prims + 255) / 256, bin_split(L)), 256, 0, stream>>>(
				L->num_prims, L->geom, L->shade, L->passes, nullptr, nullptr);
		}
		if (L->num_tmem_passes)
		{
			rdp::k_tmem_apply<<<L->num_uploads, 256, 0, stream>>>(L->passes, L->tmem_pass_list, L->num_tmem_passes,
			                                                      L->uploads, L->tmem_keep);
			rdp::k_tmem_carry<<<dim3(2048 / 32, L->num_tmem_passes), rdp::TMEM_CARRY_WARPS * 32, 0, stream>>>(
				L->passes, L->tmem_carry_list, L->tmem_keep);
		}
		if (L->num_prims && L->num_tile_items)
		{
			constexpr uint32_t per_cta = rdp::FILL_THREADS / 32 * rdp::FILL_TILES;
			rdp::k_fill<<<(L->num_tile_items + per_cta - 1) / per_cta, rdp::FILL_THREADS, 0, stream>>>(
				L->passes, L->num_passes, L->num_tile_items, L->geom, L->shade);
		}
		return cudaGetLastError();
	}
	const bool raster = L->num_prims && L->num_tile_items;
	// TMEM on the side stream: the kernels up to pair expansion read no TMEM snapshot.
	const bool side = raster && L->num_tmem_passes && L->side_stream && L->fork_event && L->join_event;
	if (side)
	{
		cudaError_t e = cudaEventRecord(L->fork_event, stream);
		if (e == cudaSuccess) e = cudaStreamWaitEvent(L->side_stream, L->fork_event, 0);
		if (e != cudaSuccess) return e;
		rdp::k_tmem_apply<<<L->num_uploads, 256, 0, L->side_stream>>>(L->passes, L->tmem_pass_list, L->num_tmem_passes,
		                                                               L->uploads, L->tmem_keep);
		rdp::k_tmem_carry<<<dim3(2048 / 32, L->num_tmem_passes), rdp::TMEM_CARRY_WARPS * 32, 0, L->side_stream>>>(
			L->passes, L->tmem_carry_list, L->tmem_keep);
		e = cudaEventRecord(L->join_event, L->side_stream);
		if (e != cudaSuccess) return e;
	}
	if (L->num_prims)
	{
		rdp::k_prim_setup<<<(L->num_prims + 127) / 128, 128, 0, stream>>>(L->prims_in, L->num_prims, L->words,
		                                                                   L->state_blocks, L->passes, L->num_passes,
		                                                                   L->geom, L->attr, L->shade,
		                                                                   L->sched && (L->sched->order_enabled ||
		                                                                                L->sched->train_enabled)
		                                                                       ? L->sched->featbits
		                                                                       : nullptr);
		uint32_t *prim_pairs = L->shade_list && L->num_tile_items ? L->prim_pairs : nullptr;
		rdp::k_bin<<<dim3((L->num_prims + 255) / 256, prim_pairs ? 1u : bin_split(L)), 256, 0, stream>>>(
			L->num_prims, L->geom, L->shade, L->passes, L->tile_counts, prim_pairs);
		// Span rows only when the pair path follows (k_scan resets their counter).
		if (L->num_tile_items && L->spans)
		{
			const uint32_t chunk = std::min<uint32_t>(
				std::max<uint32_t>(L->num_prims / (4u * std::max<uint32_t>(L->num_sms, 1u)), 1u), rdp::SPAN_THREADS / 2);
			rdp::k_span<<<(L->num_prims + chunk - 1) / chunk, rdp::SPAN_THREADS, 0, stream>>>(
				L->num_prims, L->geom, L->attr, L->shade, L->passes, static_cast<rdp::SpanRow *>(L->spans),
				L->span_capacity, L->prim_rows, reinterpret_cast<unsigned long long *>(L->ctrl + 6), chunk);
		}
	}
	if (L->num_tmem_passes && !side)
	{
		rdp::k_tmem_apply<<<L->num_uploads, 256, 0, stream>>>(L->passes, L->tmem_pass_list, L->num_tmem_passes,
		                                                      L->uploads, L->tmem_keep);
		rdp::k_tmem_carry<<<dim3(2048 / 32, L->num_tmem_passes), rdp::TMEM_CARRY_WARPS * 32, 0, stream>>>(
			L->passes, L->tmem_carry_list, L->tmem_keep);
	}
	if (raster)
	{
		// The primitive scan (primitive-major shading order) rides in the tile scan's launches.
		const uint32_t scan_prims = L->shade_list ? L->num_prims : 0u;
		// Without a span buffer every launch takes k_raster (capacity 0 rows).
		const uint2 capacity = make_uint2(L->pair_capacity, L->spans ? L->span_capacity : 0u);
		if (multi_cta_scan(L))
		{
			const uint32_t nb = (L->num_tile_items + rdp::SCAN_TILE - 1) / rdp::SCAN_TILE;
			const uint32_t nbp = (scan_prims + rdp::SCAN_TILE - 1) / rdp::SCAN_TILE;
			rdp::k_scan_reduce<<<nb + nbp, rdp::SCAN_THREADS, 0, stream>>>(L->num_tile_items, L->tile_counts,
			                                                               L->scan_blocks, nb, scan_prims,
			                                                               L->prim_pairs, L->prim_scan_blocks);
			rdp::k_scan_top<<<1, 1024, 0, stream>>>(nb, L->scan_blocks, L->num_tile_items, L->pair_offsets, L->ctrl,
			                                        capacity, L->pair_log, L->log_slot, L->shade_queues,
			                                        L->num_shade_queues, nbp, L->prim_scan_blocks);
			rdp::k_scan_down<<<nb + nbp, rdp::SCAN_THREADS, 0, stream>>>(
				L->num_tile_items, L->tile_counts, L->scan_blocks, L->pair_offsets, L->nonempty_tiles, nb, scan_prims,
				L->prim_pairs, L->prim_scan_blocks, L->prim_offsets);
		}
		else
			rdp::k_scan<<<1, 1024, 0, stream>>>(L->num_tile_items, L->tile_counts, L->pair_offsets, L->nonempty_tiles,
			                                    L->ctrl, capacity, L->pair_log, L->log_slot, L->shade_queues,
			                                    L->num_shade_queues, scan_prims, L->prim_pairs, L->prim_offsets);
		const bool sched = L->sched && (L->sched->order_enabled || L->sched->train_enabled);
		rdp::k_expand<<<(L->num_tile_items * 32 + 255) / 256, 256, 0, stream>>>(
			L->passes, L->num_passes, L->num_tile_items, L->pair_offsets, L->ctrl, L->pairs,
			sched ? L->sched->featbits : nullptr, sched ? L->sched->features : nullptr,
			sched && L->sched->train_enabled && L->tile_cycles, L->prim_offsets, L->prim_pairs, L->shade_list);
		if (side)
		{
			const cudaError_t e = cudaStreamWaitEvent(stream, L->join_event, 0);
			if (e != cudaSuccess) return e;
		}
		// Inside a stream capture the events become record nodes of the graph.
		cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
		if ((L->shade_events[0] || L->blend_events[0]) && cudaStreamIsCapturing(stream, &capture) != cudaSuccess)
			return cudaGetLastError();
		const unsigned ev_flags = capture == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u;
		if (L->shade_events[0]) cudaEventRecordWithFlags(L->shade_events[0], stream, ev_flags);
		const uint32_t sv = L->shade_variant < RDP_SHADE_VARIANTS ? L->shade_variant : 0;
		const ShadeKernel shade_kernel = kShadeVariants[sv];
		shade_kernel<<<L->shade_ctas, rdp::SHADE_THREADS, 0, stream>>>(
			L->passes, L->num_passes, L->pairs, L->ctrl, L->geom, L->attr, L->shade, L->tilesets, L->scratch,
			L->shade_list, L->shade_queues, L->num_shade_queues, L->shade_queue_min,
			static_cast<const rdp::SpanRow *>(L->spans), L->prim_rows);
		if (L->shade_events[1]) cudaEventRecordWithFlags(L->shade_events[1], stream, ev_flags);
		const uint32_t tile_ctas = std::min<uint32_t>(L->num_tile_items, L->blend_ctas);
		const uint32_t *order = L->tile_order;
		if (L->sched && (L->sched->order_enabled || L->sched->train_enabled))
		{
			// Features + predictions (also the training inputs), then the longest-first order.
			cudaError_t e = rdp_sched_launch_order(L->sched, L->pair_offsets, L->ctrl, L->nonempty_tiles,
			                                       L->blend_ctas / 4 + 1, stream);
			if (e != cudaSuccess) return e;
			if (L->sched->order_enabled) order = L->sched->order;
		}
		if (L->blend_events[0]) cudaEventRecordWithFlags(L->blend_events[0], stream, ev_flags);
		if (L->blend_kernel)
			rdp::k_blend<<<tile_ctas, rdp::SHADE_THREADS, 0, stream>>>(
				L->passes, L->num_passes, L->pair_offsets, L->pairs, L->ctrl, L->nonempty_tiles, L->shade, L->scratch,
				order, L->tile_cycles);
		else
			rdp::k_blend_lookahead<<<tile_ctas, rdp::SHADE_THREADS, 0, stream>>>(
				L->passes, L->num_passes, L->pair_offsets, L->pairs, L->ctrl, L->nonempty_tiles, L->shade, L->scratch,
				order, L->tile_cycles);
		if (L->blend_events[1]) cudaEventRecordWithFlags(L->blend_events[1], stream, ev_flags);
		if (L->sched && L->sched->train_enabled && L->tile_cycles)
		{
			cudaError_t e = rdp_sched_launch_train(L->sched, L->ctrl, L->nonempty_tiles, L->tile_cycles,
			                                       L->blend_ctas / 8 + 1, stream);
			if (e != cudaSuccess) return e;
		}
		rdp::k_raster<<<tile_ctas, rdp::RASTER_THREADS, 0, stream>>>(
			L->passes, L->num_passes, L->num_tile_items, L->geom, L->attr, L->shade, L->tilesets, L->ctrl);
	}
	return cudaGetLastError();
}

// ============================================================================ allocation-free TMEM update
// A variant of k_tmem_apply / k_tmem_carry for callers that cannot allocate device memory: the
// per-upload "word kept" bitmask lives in this file-scope array instead of a cudaMalloc'd buffer.
// It is fully rewritten for every upload a call applies before it is read, so it needs no clearing.
#include "../../include/rdp_cuda.h"
#include <mutex>

static_assert(sizeof(rdp_tmem_upload) == sizeof(RdpUpload), "rdp_tmem_upload must mirror RdpUpload");

static __device__ __align__(256) uint32_t g_noalloc_tmem_keep[RDP_NOALLOC_MAX_UPLOADS * 64];

namespace rdp {
struct NoallocTmem
{
	const uint8_t *rdram;
	uint32_t rdram_size;
	uint16_t *tmem;
	uint16_t *snapshots;
	uint32_t count;
};

__global__ void k_tmem_apply_noalloc(NoallocTmem a, const RdpUpload *__restrict__ uploads, uint32_t *__restrict__ keep_bits)
{
	RdpPass ps = {};
	ps.rdram = const_cast<uint8_t *>(a.rdram);
	ps.rdram_size = a.rdram_size;
	uint32_t u = blockIdx.x;
	if (u >= a.count) return;
	RdpUpload info = uploads[u];
	uint16_t *dst = a.snapshots + size_t(u + 1) * 2048;
	uint32_t *keep = keep_bits + size_t(u) * 64;
	for (int gid = threadIdx.x; gid < 2048; gid += blockDim.x)
	{
		int idx = gid ^ 1;
		bool upper = idx >= 0x400;
		uint32_t v = 0;
		bool wrote;
		if (info.mode == 1) wrote = tmem_lut(ps, info, idx, v);
		else
		{
			bool yuv = info.tmem_fmt == 1;
			if (info.tmem_size == 3 || yuv) wrote = tmem_32(ps, info, idx & 0x3ff, upper, yuv, v);
			else wrote = tmem_16(ps, info, idx, v);
		}
		if (wrote) dst[gid] = uint16_t(v);
		unsigned m = __ballot_sync(0xffffffffu, !wrote);
		if ((threadIdx.x & 31) == 0) keep[gid >> 5] = m;
	}
}

__global__ void k_tmem_carry_noalloc(NoallocTmem a, const uint32_t *__restrict__ keep_bits)
{
	int gid = blockIdx.x * blockDim.x + threadIdx.x;
	if (gid >= 2048) return;
	uint16_t value = a.tmem[gid];
	a.snapshots[gid] = value;
	for (uint32_t u = 0; u < a.count; u++)
	{
		size_t at = size_t(u + 1) * 2048 + gid;
		uint16_t written = a.snapshots[at];
		bool keep_prev = (keep_bits[u * 64 + (gid >> 5)] >> (gid & 31)) & 1u;
		if (keep_prev) a.snapshots[at] = value;
		value = keep_prev ? value : written;
	}
	a.tmem[gid] = value;
}
} // namespace rdp

namespace {
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
uint32_t *g_noalloc_keep_ptr[kNoallocMaxDevices] = {};
}

extern "C" int rdp_tmem_update_noalloc(const rdp_tmem_upload *uploads, uint32_t num_uploads, const uint8_t *rdram,
                                       uint32_t rdram_size, uint16_t *tmem, uint16_t *snapshots, void *stream)
{
	if (num_uploads > RDP_NOALLOC_MAX_UPLOADS) return RDP_ERR_TOO_LARGE;
	if (!rdram || !tmem || !snapshots || (num_uploads && !uploads)) return RDP_ERR_INVALID;
	if (!rdram_size || (rdram_size & (rdram_size - 1))) return RDP_ERR_INVALID;
	int device = 0;
	if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kNoallocMaxDevices) return RDP_ERR_DEVICE;
	uint32_t *keep;
	{
		// Per-device set-up, with that device current: the host-side name of the array is not a
		// device address, so ask the runtime for the device address once.
		std::lock_guard<std::mutex> hold(g_noalloc_mutex);
		if (!g_noalloc_keep_ptr[device])
		{
			void *ptr = nullptr;
			if (cudaGetSymbolAddress(&ptr, g_noalloc_tmem_keep) != cudaSuccess || !ptr)
			{
				cudaGetLastError();
				return RDP_ERR_DEVICE;
			}
			g_noalloc_keep_ptr[device] = static_cast<uint32_t *>(ptr);
		}
		keep = g_noalloc_keep_ptr[device];
	}
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	rdp::NoallocTmem a = { rdram, rdram_size, tmem, snapshots, num_uploads };
	if (num_uploads)
		rdp::k_tmem_apply_noalloc<<<num_uploads, 256, 0, s>>>(a, reinterpret_cast<const RdpUpload *>(uploads), keep);
	rdp::k_tmem_carry_noalloc<<<2048 / 32, 32, 0, s>>>(a, keep);
	return cudaGetLastError() == cudaSuccess ? RDP_OK : RDP_ERR_DEVICE;
}
