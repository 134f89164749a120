/*
 * Video Interface (scanout) kernels for sm_103a.
 *
 *   k_vi_fetch : one thread per pixel of the filtered fetch image.  Reads the
 *                framebuffer pixel and its neighbours straight from RDRAM
 *                (extract_vram.comp) and applies the AA filter (second lowest /
 *                highest of the full-coverage neighbours) or the dither
 *                reconstruction filter (vi_fetch.frag), with the fetch-bug layer.
 *   k_vi_divot : horizontal 3-tap median where any tap lacks full coverage
 *                (vi_divot.frag).
 *   k_vi_scale : one thread per output pixel: XStart/XAdd, YStart/YAdd sampling,
 *                5-bit bilinear, serrate, gamma table or gamma dither
 *                (vi_scale.frag), then the previous-frame blend for pixels the
 *                current frame leaves empty (video_interface.cpp:912-988).
 * Images are RGBA8 words (r | g << 8 | b << 16 | a << 24); reads outside an image
 * return 0.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include "vi.h"

namespace rdpvi {

__device__ uint8_t g_gamma[256 + 256 * 64];

__device__ __forceinline__ uint32_t pack(uint32_t r, uint32_t g, uint32_t b, uint32_t a)
{
	return (r & 0xff) | ((g & 0xff) << 8) | ((b & 0xff) << 16) | ((a & 0xff) << 24);
}
__device__ __forceinline__ uint32_t ch(uint32_t c, int i) { return (c >> (8 * i)) & 0xff; }

// extract_vram.comp: one framebuffer pixel with its 3-bit coverage; an upscaled pixel reads its
// sample slice (extract_vram.comp:58-67).
__device__ uint32_t fetch_vram(const RdpViParams &p, int cx, int cy)
{
	const int sl = p.scale_log2, m = (1 << sl) - 1;
	const int slice = ((cy & m) << sl) + (cx & m);
	cx >>= sl;
	cy >>= sl;
	int lin = cy * p.fb_width + cx + p.fb_offset;
	uint32_t r, g, b, a;
	if (p.is_8888)
	{
		lin &= int((p.rdram_size >> 2) - 1);
		lin += slice * int(p.rdram_size >> 2);
		uint32_t w = *reinterpret_cast<const uint32_t *>(p.rdram + size_t(lin) * 4);
		r = (w >> 24) & 0xff; g = (w >> 16) & 0xff; b = (w >> 8) & 0xff; a = (w >> 5) & 7;
	}
	else
	{
		lin &= int((p.rdram_size >> 1) - 1);
		lin += slice * int(p.rdram_size >> 1);
		uint32_t w = *reinterpret_cast<const uint16_t *>(p.rdram + size_t(lin ^ 1) * 2);
		uint32_t hw = p.hidden[lin];
		r = (w >> 8) & 0xf8; g = (w >> 3) & 0xf8; b = (w << 2) & 0xf8; a = ((w & 1) << 2) | hw;
	}
	if (!p.fetch_aa) a = 7;
	return pack(r, g, b, a);
}

__device__ __forceinline__ void check_neighbor(uint32_t c, uint32_t lo[3], uint32_t hi[3], uint32_t slo[3], uint32_t shi[3])
{
	if (ch(c, 3) == 7)
	{
#pragma unroll
		for (int i = 0; i < 3; i++)
		{
			uint32_t v = ch(c, i);
			slo[i] = min(slo[i], max(v, lo[i]));
			shi[i] = max(shi[i], min(v, hi[i]));
			lo[i] = min(v, lo[i]);
			hi[i] = max(v, hi[i]);
		}
	}
}

__global__ void k_vi_fetch(RdpViParams p)
{
	int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= p.aa_w || y >= p.aa_h) return;
	// The fetch image is offset by (-2 or -3, -2) from the framebuffer; the filter reads at (+2, +2).
	int fx = x + 2 + (p.divot ? -3 : -2), fy = y + 2 - 2;
	uint32_t mid = fetch_vram(p, fx, fy);
	uint32_t col[3], bug[3];
	uint32_t ma = ch(mid, 3);
	if (ma != 7)
	{
		uint32_t lo[3], hi[3], slo[3], shi[3];
#pragma unroll
		for (int i = 0; i < 3; i++) lo[i] = hi[i] = slo[i] = shi[i] = ch(mid, i);
		uint32_t lu = fetch_vram(p, fx - 1, fy - 1), ru = fetch_vram(p, fx + 1, fy - 1);
		uint32_t tl = fetch_vram(p, fx - 2, fy), tr = fetch_vram(p, fx + 2, fy);
		uint32_t ld = fetch_vram(p, fx - 1, fy + 1), rd = fetch_vram(p, fx + 1, fy + 1);
		check_neighbor(lu, lo, hi, slo, shi);
		check_neighbor(ru, lo, hi, slo, shi);
		check_neighbor(tl, lo, hi, slo, shi);
		check_neighbor(tr, lo, hi, slo, shi);
		uint32_t lob[3], hib[3], slob[3], shib[3];
#pragma unroll
		for (int i = 0; i < 3; i++) { lob[i] = lo[i]; hib[i] = hi[i]; slob[i] = slo[i]; shib[i] = shi[i]; }
		check_neighbor(ld, lo, hi, slo, shi);
		check_neighbor(rd, lo, hi, slo, shi);
		if (p.fetch_bug)
		{
			check_neighbor(tl, lob, hib, slob, shib);
			check_neighbor(tr, lob, hib, slob, shib);
#pragma unroll
			for (int i = 0; i < 3; i++)
			{
				uint32_t m = ch(mid, i);
				if (m == lo[i]) slo[i] = lo[i];
				if (m == hi[i]) shi[i] = hi[i];
				if (m == lob[i]) slob[i] = lob[i];
				if (m == hib[i]) shib[i] = hib[i];
			}
		}
		uint32_t coeff = 7u - ma;
#pragma unroll
		for (int i = 0; i < 3; i++)
		{
			uint32_t m = ch(mid, i);
			col[i] = (m + (((slo[i] + shi[i] - (m << 1)) * coeff + 4u) >> 3)) & 0xff;
			bug[i] = (m + (((slob[i] + shib[i] - (m << 1)) * coeff + 4u) >> 3)) & 0xff;
		}
	}
	else if (p.dither_filter)
	{
		int tc[3], acc[3] = { 0, 0, 0 }, accb[3];
#pragma unroll
		for (int i = 0; i < 3; i++) tc[i] = int(ch(mid, i) >> 3);
		for (int yy = -1; yy <= 0; yy++)
			for (int xx = -1; xx <= 1; xx++)
			{
				uint32_t c = fetch_vram(p, fx + xx, fy + yy);
#pragma unroll
				for (int i = 0; i < 3; i++) acc[i] += min(max(int(ch(c, i) >> 3) - tc[i], -1), 1);
			}
#pragma unroll
		for (int i = 0; i < 3; i++) accb[i] = acc[i];
		const int dxs[3] = { -1, 1, 0 };
		for (int k = 0; k < 3; k++)
		{
			uint32_t c = fetch_vram(p, fx + dxs[k], fy + 1);
#pragma unroll
			for (int i = 0; i < 3; i++) acc[i] += min(max(int(ch(c, i) >> 3) - tc[i], -1), 1);
		}
		for (int k = 0; k < 2; k++)
		{
			uint32_t c = fetch_vram(p, fx + (k ? 1 : -1), fy);
#pragma unroll
			for (int i = 0; i < 3; i++) accb[i] += min(max(int(ch(c, i) >> 3) - tc[i], -1), 1);
		}
#pragma unroll
		for (int i = 0; i < 3; i++)
		{
			col[i] = uint32_t(int(ch(mid, i) & 0xf8) + acc[i]);
			bug[i] = uint32_t(int(ch(mid, i) & 0xf8) + accb[i]);
		}
	}
	else
	{
#pragma unroll
		for (int i = 0; i < 3; i++) col[i] = bug[i] = ch(mid, i);
	}
	size_t plane = size_t(p.aa_w) * p.aa_h;
	p.aa[size_t(y) * p.aa_w + x] = pack(col[0], col[1], col[2], ma);
	if (p.fetch_bug) p.aa[plane + size_t(y) * p.aa_w + x] = pack(bug[0], bug[1], bug[2], ma);
}

__device__ __forceinline__ uint32_t img_get(const uint32_t *img, int w, int h, int x, int y, int layer)
{
	if (x < 0 || y < 0 || x >= w || y >= h) return 0;
	return img[(size_t(layer) * h + y) * w + x];
}

__device__ __forceinline__ uint32_t median3(uint32_t a, uint32_t b, uint32_t c)
{
	if (a < b) { uint32_t t = a; a = b; b = t; }
	if (b < c) { uint32_t t = b; b = c; c = t; }
	if (a < b) { uint32_t t = a; a = b; b = t; }
	return b;
}

__global__ void k_vi_divot(RdpViParams p)
{
	int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
	int layer = blockIdx.z;
	if (x >= p.dv_w || y >= p.dv_h) return;
	uint32_t le = img_get(p.aa, p.aa_w, p.aa_h, x, y, layer);
	uint32_t mi = img_get(p.aa, p.aa_w, p.aa_h, x + 1, y, layer);
	uint32_t ri = img_get(p.aa, p.aa_w, p.aa_h, x + 2, y, layer);
	uint32_t o;
	if ((ch(le, 3) & ch(mi, 3) & ch(ri, 3)) == 7)
		o = mi;
	else
		o = pack(median3(ch(le, 0), ch(mi, 0), ch(ri, 0)), median3(ch(le, 1), ch(mi, 1), ch(ri, 1)),
		         median3(ch(le, 2), ch(mi, 2), ch(ri, 2)), ch(mi, 3));
	p.dv[(size_t(layer) * p.dv_h + y) * p.dv_w + x] = o;
}

__device__ __forceinline__ bool in_rect(int x, int y, int rx, int ry, int rw, int rh, int cx, int cy)
{
	rx -= cx;
	ry -= cy;
	if (rx < 0) { rw += rx; rx = 0; }
	if (ry < 0) { rh += ry; ry = 0; }
	if (rw <= 0 || rh <= 0) return false;
	return x >= rx && x < rx + rw && y >= ry && y < ry + rh;
}

__device__ __forceinline__ uint32_t vi_lerp(uint32_t a, uint32_t b, uint32_t l) { return (a + (((b - a) * l + 16u) >> 5)) & 0xff; }

__global__ void k_vi_scale(RdpViParams p)
{
	int fx = blockIdx.x * blockDim.x + threadIdx.x, fy = blockIdx.y * blockDim.y + threadIdx.y;
	if (fx >= p.out_w || fy >= p.out_h) return;
	uint32_t result = 0;
	bool written = false;
	if (p.draw && in_rect(fx, fy, p.h_start, p.v_start, p.h_res, p.v_res, p.crop_left, p.crop_top))
	{
		int cx = fx + p.crop_left, cy = fy + p.crop_top;
		int li_index = min(cy >> p.info_y_shift, RDP_VI_MAX_LINES - 1);
		RdpViLine li = p.lines[li_index];
		cy -= p.v_start;
		if (!(cx < li.h_start_clamp || cx >= li.h_end_clamp || ((cy & p.serrate_mask) != p.serrate_select)))
		{
			cx -= li.h_start;
			cy >>= p.serrate_shift;
			uint32_t seed = 0;
			if (p.gamma_dither)
			{
				const uint32_t P = 1103515245u;
				uint32_t s0 = uint32_t(cx), s1 = uint32_t(cy), s2 = p.frame_count;
#pragma unroll
				for (int k = 0; k < 3; k++)
				{
					uint32_t n0 = ((s0 >> 8) ^ s1) * P, n1 = ((s1 >> 8) ^ s2) * P, n2 = ((s2 >> 8) ^ s0) * P;
					s0 = n0; s1 = n1; s2 = n2;
				}
				seed = (s0 >> 16) & 0xffff;
			}
			int x = cx * li.x_add + li.x_start;
			int y = (cy - li.y_base) * li.y_add + li.y_start;
			int bx = x >> 10, by = y >> 10;
			uint32_t c00 = img_get(p.dv, p.dv_w, p.dv_h, bx, by, 0);
			int bug_offset = 0;
			if (p.fetch_bug)
			{
				int prev_y = (y - p.init_y_add) >> 10, next_y = (y + p.init_y_add) >> 10;
				if (cy != 0 && by == prev_y && by != next_y) bug_offset = 1;
			}
			uint32_t res[3] = { ch(c00, 0), ch(c00, 1), ch(c00, 2) };
			if (p.scale_aa)
			{
				uint32_t xf = uint32_t((x >> 5) & 31), yf = uint32_t((y >> 5) & 31);
				uint32_t c10 = img_get(p.dv, p.dv_w, p.dv_h, bx + 1, by, 0);
				uint32_t c01 = img_get(p.dv, p.dv_w, p.dv_h, bx, by + 1, bug_offset);
				uint32_t c11 = img_get(p.dv, p.dv_w, p.dv_h, bx + 1, by + 1, bug_offset);
#pragma unroll
				for (int i = 0; i < 3; i++)
				{
					uint32_t a = vi_lerp(ch(c00, i), ch(c01, i), yf);
					uint32_t b = vi_lerp(ch(c10, i), ch(c11, i), yf);
					res[i] = vi_lerp(a, b, xf);
				}
			}
			if (p.gamma)
			{
#pragma unroll
				for (int i = 0; i < 3; i++)
				{
					uint32_t idx = res[i];
					if (p.gamma_dither)
					{
						uint32_t d = i == 0 ? (seed & 0x3f) : i == 1 ? ((seed >> 6) & 0x3f) : (((seed >> 9) & 0x38) | (seed & 7));
						idx = (res[i] << 6) + d + 256u;
					}
					res[i] = g_gamma[min(idx, 256u + 256u * 64u - 1u)];
				}
			}
			else if (p.gamma_dither)
			{
#pragma unroll
				for (int i = 0; i < 3; i++) res[i] = min(res[i] + ((seed >> i) & 1u), 0xffu);
			}
			result = pack(res[0], res[1], res[2], 255);
			written = true;
		}
	}
	if (!written && p.blend_prev)
	{
		bool blend;
		if (p.degenerate)
			blend = p.h_res > 0 && in_rect(fx, fy, p.h_start, 0, p.h_res, p.prev_h, p.crop_left, p.crop_top);
		else
			blend = (p.h_res > 0 && p.v_start > 0 && in_rect(fx, fy, p.h_start, 0, p.h_res, p.v_start, p.crop_left, p.crop_top)) ||
			        (p.h_res_clamp > 0 && p.v_res > 0 &&
			         in_rect(fx, fy, p.h_start_clamp, p.v_start, p.h_res_clamp, p.v_res, p.crop_left, p.crop_top)) ||
			        (p.h_res > 0 && p.prev_h > p.v_start + p.v_res &&
			         in_rect(fx, fy, p.h_start, p.v_start + p.v_res, p.h_res, p.prev_h - (p.v_start + p.v_res), p.crop_left,
			                 p.crop_top));
		if (blend)
		{
			uint32_t pv = img_get(p.prev, p.prev_w, p.prev_h, fx, fy, 0);
			result = ch(pv, 3) == 255 ? (pv & 0x00ffffffu) : 0u;
		}
	}
	p.out[size_t(fy) * p.out_w + fx] = result;
}

} // namespace rdpvi

extern "C" cudaError_t rdp_vi_init_tables(void)
{
	static uint8_t g[256 + 256 * 64];
	auto isq = [](int v) {
		int r = 0;
		while ((r + 1) * (r + 1) <= v) r++;
		return r;
	};
	for (int i = 0; i < 256; i++) g[i] = uint8_t(isq(i * 256) & ~1);
	for (int i = 0; i < 256 * 64; i++) g[256 + i] = uint8_t(isq(i * 4) & ~1);
	return cudaMemcpyToSymbol(rdpvi::g_gamma, g, sizeof(g));
}

namespace rdpvi {
__global__ void k_vi_half(const uint32_t *__restrict__ src, int w, uint32_t *__restrict__ dst, int hw, int hh)
{
	const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= hw || y >= hh) return;
	const uint32_t a = src[size_t(2 * y) * w + 2 * x], b = src[size_t(2 * y) * w + 2 * x + 1];
	const uint32_t c = src[size_t(2 * y + 1) * w + 2 * x], d = src[size_t(2 * y + 1) * w + 2 * x + 1];
	uint32_t o = 0;
#pragma unroll
	for (int i = 0; i < 4; i++) o |= ((ch(a, i) + ch(b, i) + ch(c, i) + ch(d, i) + 2) >> 2) << (8 * i);
	dst[size_t(y) * hw + x] = o;
}
} // namespace rdpvi

extern "C" cudaError_t rdp_vi_downscale(const uint32_t *src, int32_t w, int32_t h, uint32_t *dst, cudaStream_t stream)
{
	const int hw = w / 2, hh = h / 2;
	if (hw <= 0 || hh <= 0) return cudaSuccess;
	rdpvi::k_vi_half<<<dim3((hw + 15) / 16, (hh + 7) / 8), dim3(16, 8), 0, stream>>>(src, w, dst, hw, hh);
	return cudaGetLastError();
}

extern "C" cudaError_t rdp_vi_launch(const RdpViParams *p, cudaStream_t stream)
{
	dim3 blk(16, 8);
	if (!p->degenerate && p->aa_w > 0 && p->aa_h > 0)
	{
		rdpvi::k_vi_fetch<<<dim3((p->aa_w + 15) / 16, (p->aa_h + 7) / 8), blk, 0, stream>>>(*p);
		if (p->divot)
			rdpvi::k_vi_divot<<<dim3((p->dv_w + 15) / 16, (p->dv_h + 7) / 8, p->fetch_bug ? 2 : 1), blk, 0, stream>>>(*p);
	}
	rdpvi::k_vi_scale<<<dim3((p->out_w + 15) / 16, (p->out_h + 7) / 8), blk, 0, stream>>>(*p);
	return cudaGetLastError();
}
