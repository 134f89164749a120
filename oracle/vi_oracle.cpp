/*
 * CPU ORACLE for the Video Interface (scanout) -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, in scalar C++, the reference's VI path at 1x scale:
 *   - register decode:  parallel-rdp/video_interface.cpp:177-367 (decode_vi_registers)
 *   - per-scanline registers: video_interface.cpp:1102-1213
 *   - frame logic:      video_interface.cpp:1215-1426 (scanout)
 *   - VRAM fetch:       parallel-rdp/shaders/extract_vram.comp
 *   - AA / dither filter (with the fetch-bug layer): shaders/vi_fetch.frag
 *   - divot median:     shaders/vi_divot.frag
 *   - scale, gamma, gamma dither: shaders/vi_scale.frag
 *   - previous-frame blend: video_interface.cpp:912-988, shaders/vi_blend_fields.frag
 * The intermediate images are plain arrays; texel fetches outside an image read 0.
 * It reads the oracle renderer's RDRAM / hidden RDRAM (rdp_oracle.cpp) through a
 * small accessor interface.
 */
#include <stdint.h>
#include <string.h>
#include <math.h>
#include <algorithm>
#include <vector>
#include <functional>

namespace {

enum
{
	VI_TYPE_MASK = 3, VI_TYPE_5551 = 2, VI_TYPE_8888 = 3,
	VI_GAMMA_DITHER = 1 << 2, VI_GAMMA = 1 << 3, VI_DIVOT = 1 << 4, VI_SERRATE = 1 << 6,
	VI_AA_MASK = 3 << 8, VI_DITHER_FILTER = 1 << 16, VI_META_AA = 1 << 17, VI_META_SCALE = 1 << 18
};
constexpr int V_SYNC_NTSC = 525, H_OFFSET_NTSC = 108, H_OFFSET_PAL = 128, V_OFFSET_NTSC = 34, V_OFFSET_PAL = 44;
constexpr int V_RES_NTSC = 480, V_RES_PAL = 576, SCANOUT_WIDTH = 640;
constexpr int V_END_PAL = (V_OFFSET_PAL + V_RES_PAL) | 1, V_END_NTSC = (V_OFFSET_NTSC + V_RES_NTSC) | 1;
constexpr int V_END_MAX = V_END_PAL > V_END_NTSC ? V_END_PAL : V_END_NTSC;
constexpr int MAX_OUTPUT_SCANLINES = V_RES_PAL >> 1;

struct Line
{
	int h_start, h_start_clamp, h_end_clamp, x_start, x_add, y_start, y_add, y_base;
};

struct Regs
{
	int vi_width, vi_offset, v_current_line, v_start, init_y_add, v_res, is_pal, max_x, max_y;
	int h_start, h_res, h_start_clamp, h_res_clamp;
	uint32_t status;
};

struct Img
{
	int w = 0, h = 0, layers = 1;
	std::vector<uint8_t> px; // RGBA per pixel
	void init(int w_, int h_, int l)
	{
		w = w_; h = h_; layers = l;
		px.assign(size_t(w) * h * l * 4, 0);
	}
	uint8_t *at(int x, int y, int l) { return &px[((size_t(l) * h + y) * w + x) * 4]; }
	void get(int x, int y, int l, uint32_t c[4]) const
	{
		if (x < 0 || y < 0 || x >= w || y >= h || l >= layers) { c[0] = c[1] = c[2] = c[3] = 0; return; }
		const uint8_t *p = &px[((size_t(l) * h + y) * w + x) * 4];
		for (int i = 0; i < 4; i++) c[i] = p[i];
	}
};

static inline int isqrt_int(int v) { int r = int(sqrt(double(v))); while (r * r > v) r--; while ((r + 1) * (r + 1) <= v) r++; return r; }

} // namespace

struct ViOracle
{
	uint32_t regs[14] = {};
	// Per-scanline state (video_interface.hpp PerScanlineRegisterState).
	uint32_t ps_flags = 0;
	bool ps_ended = false;
	unsigned ps_line = 0;
	uint32_t hs_latched = 0, xs_latched = 0;
	uint32_t hs_line[V_END_MAX] = {}, xs_line[V_END_MAX] = {};

	bool previous_frame_blank = false;
	uint32_t frame_count = 0, last_valid_frame_count = 0;
	Img prev;
	bool have_prev = false;
	uint8_t gamma[256 + 256 * 64];

	ViOracle()
	{
		for (int i = 0; i < 256; i++) gamma[i] = uint8_t(isqrt_int(i * 256) & ~1);
		for (int i = 0; i < 256 * 64; i++) gamma[256 + i] = uint8_t(isqrt_int(i * 4) & ~1);
	}

	Regs decode(Line *lines)
	{
		Regs r = {};
		r.status = regs[0];
		r.vi_width = regs[2] & 0xfff;
		r.vi_offset = regs[1] & 0xffffff;
		r.v_current_line = regs[4] & 1;
		r.v_start = (regs[10] >> 16) & 0x3ff;
		int y_start = (regs[13] >> 16) & 0xfff;
		int y_add = regs[13] & 0xfff;
		r.init_y_add = y_add;
		int v_end = regs[10] & 0x3ff;
		int v_sync = regs[6] & 0x3ff;
		r.is_pal = unsigned(v_sync) > (V_SYNC_NTSC + 25);
		int v_end_max = r.is_pal ? V_END_PAL : V_END_NTSC;
		if (v_end > v_end_max) v_end = v_end_max;
		if (r.v_start > v_end_max) r.v_start = v_end_max;
		int v_start_offset = r.is_pal ? V_OFFSET_PAL : V_OFFSET_NTSC;
		r.v_res = (v_end - r.v_start) >> 1;
		r.v_start = (r.v_start - v_start_offset) / 2;
		if (r.v_start < 0)
		{
			y_start -= y_add * r.v_start;
			r.v_start = 0;
		}
		r.v_res = std::min(r.v_res, MAX_OUTPUT_SCANLINES - r.v_start);
		int hsc_lo = INT32_MAX, hec_hi = 0, hs_lo = INT32_MAX, he_hi = 0;
		r.max_x = 0;
		bool degenerate_y = r.v_res <= 0;
		if (lines)
		{
			if (degenerate_y)
				for (int i = 0; i < MAX_OUTPUT_SCANLINES; i++) lines[i] = {};
			else
			{
				for (int i = 0; i < r.v_start; i++) lines[i] = {};
				for (int i = r.v_start + r.v_res; i < MAX_OUTPUT_SCANLINES; i++) lines[i] = {};
			}
		}
		auto analyze = [&](int x_start, int x_add, int h_start, int h_end, Line *line) {
			bool lc = false, rc = false;
			h_start -= r.is_pal ? H_OFFSET_PAL : H_OFFSET_NTSC;
			h_end -= r.is_pal ? H_OFFSET_PAL : H_OFFSET_NTSC;
			if (h_start < 0)
			{
				x_start -= x_add * h_start;
				h_start = 0;
				lc = true;
			}
			if (h_end > SCANOUT_WIDTH)
			{
				h_end = SCANOUT_WIDTH;
				rc = true;
			}
			int hsc = h_start + (lc ? 0 : 8);
			int hec = h_end - (rc ? 0 : 7);
			int h_res = h_end - h_start;
			int max_x = (x_start + h_res * x_add) >> 10;
			r.max_x = std::max(r.max_x, max_x);
			hs_lo = std::min(hs_lo, h_start);
			he_hi = std::max(he_hi, h_end);
			hsc_lo = std::min(hsc_lo, hsc);
			hec_hi = std::max(hec_hi, hec);
			if (line) *line = { h_start, hsc, hec, x_start, x_add, y_start, y_add, 0 };
		};
		if (degenerate_y || !ps_ended)
		{
			Line li;
			analyze((regs[12] >> 16) & 0xfff, regs[12] & 0xfff, (regs[9] >> 16) & 0x3ff, regs[9] & 0x3ff, &li);
			if (lines)
				for (int i = r.v_start; i < r.v_start + r.v_res; i++) lines[i] = li;
		}
		else
		{
			for (int i = r.v_start; i < r.v_start + r.v_res; i++)
			{
				int eff = 2 * i + v_start_offset + int(r.v_current_line == 0);
				analyze((xs_line[eff] >> 16) & 0xfff, xs_line[eff] & 0xfff, (hs_line[eff] >> 16) & 0x3ff, hs_line[eff] & 0x3ff,
				        lines ? &lines[i] : nullptr);
			}
		}
		r.max_y = (y_start + r.v_res * y_add) >> 10;
		r.h_start = hs_lo;
		r.h_res = he_hi - hs_lo;
		r.h_start_clamp = hsc_lo;
		r.h_res_clamp = hec_hi - hsc_lo;
		return r;
	}

	// Options mirror ScanoutOptions (video_interface.hpp:31-81).
	struct Options
	{
		uint32_t crop_overscan_pixels, crop_rect_enable, crop_left, crop_right, crop_top, crop_bottom;
		uint32_t persist_frame_on_invalid_input, blend_previous_frame, upscale_deinterlacing;
		uint32_t vi_aa, vi_scale, vi_serrate, vi_dither_filter, vi_divot_filter, vi_gamma_dither;
		uint32_t downscale_steps;
	};

	// VideoInterface::scanout_memory_range (video_interface.cpp:369-396): the bytes the fetch reads,
	// from the registers as they are after the per-scanline state is cleared.
	void memory_range(uint32_t &offset, uint32_t &length)
	{
		const bool ended = ps_ended;
		ps_ended = false;
		Regs r = decode(nullptr);
		ps_ended = ended;
		bool divot = (r.status & VI_DIVOT) != 0;
		int aw = r.max_x + 2 + 4 + int(divot) * 2, ah = r.max_y + 1 + 4;
		if (r.vi_offset == 0 || r.h_res <= 0 || r.h_start >= SCANOUT_WIDTH)
		{
			offset = length = 0;
			return;
		}
		int pixel_size = ((r.status & VI_TYPE_MASK) | VI_TYPE_5551) == VI_TYPE_8888 ? 4 : 2;
		int off = r.vi_offset & ~(pixel_size - 1);
		off += ((divot ? -3 : -2) + -2 * r.vi_width) * pixel_size;
		offset = uint32_t(off);
		length = uint32_t((ah * r.vi_width + aw) * pixel_size);
	}

	// Returns true and fills `out` when an image is produced.  With an upscaling factor S > 1 the
	// sources are the multisampled copies (S * S slices of rdram_size / hidden bytes) and the image
	// is S times larger (video_interface.cpp:1299-1318), then halved downscale_steps times.
	// `sources` is called when the framebuffer is fetched (not for frames without an image) and
	// returns the RDRAM and hidden RDRAM to fetch from.
	bool scanout(const Options &o, const std::function<std::pair<const uint8_t *, const uint8_t *>()> &sources,
	             uint32_t rdram_size, Img &out, int S = 1)
	{
		Line lines[MAX_OUTPUT_SCANLINES];
		Regs r = decode(lines);
		ps_flags = 0;
		ps_ended = false;
		const int L = S == 8 ? 3 : S == 4 ? 2 : S == 2 ? 1 : 0;
		if (r.vi_offset == 0)
		{
			have_prev = false;
			return false;
		}
		if (!o.vi_serrate) r.status &= ~VI_SERRATE;
		bool is_aa = (r.status & VI_AA_MASK) < (2u << 8);
		bool is_bilinear = (r.status & VI_AA_MASK) < (3u << 8);
		is_aa = is_aa && o.vi_aa;
		is_bilinear = is_bilinear && o.vi_scale;
		r.status &= ~(VI_AA_MASK | VI_META_AA | VI_META_SCALE);
		if (is_aa) r.status |= VI_META_AA;
		if (is_bilinear) r.status |= VI_META_SCALE;
		if (!o.vi_gamma_dither) r.status &= ~VI_GAMMA_DITHER;
		if (!o.vi_divot_filter) r.status &= ~VI_DIVOT;
		if (!o.vi_dither_filter) r.status &= ~VI_DITHER_FILTER;
		bool is_blank = (r.status & VI_TYPE_5551) == 0;
		if (is_blank && previous_frame_blank)
		{
			frame_count++;
			have_prev = false;
			return false;
		}
		if (is_blank) have_prev = false;
		r.status |= VI_TYPE_5551;
		previous_frame_blank = is_blank;
		bool divot = (r.status & VI_DIVOT) != 0;
		if (r.h_res <= 0 || r.h_start >= SCANOUT_WIDTH)
		{
			frame_count++;
			if (o.persist_frame_on_invalid_input && (frame_count - last_valid_frame_count < 4) && have_prev)
			{
				out = prev;
				return true;
			}
			have_prev = false;
			return false;
		}
		last_valid_frame_count = frame_count;
		bool degenerate = r.h_res <= 0 || r.v_res <= 0;
		if (S > 1)
		{
			r.h_start *= S;
			r.h_start_clamp *= S;
			r.v_start *= S;
			r.h_res *= S;
			r.h_res_clamp *= S;
			r.v_res *= S;
			r.max_x = r.max_x * S + (S - 1);
			r.max_y = r.max_y * S + (S - 1);
			for (Line &li : lines)
			{
				li.h_start *= S;
				li.h_start_clamp *= S;
				li.h_end_clamp *= S;
				li.x_start *= S;
				li.y_start *= S;
				li.y_base *= S;
			}
		}
		// need_fetch_bug_emulation (video_interface.cpp:398-403).
		bool fetch_bug = r.init_y_add < 1024 && S == 1;
		bool is_8888 = (r.status & VI_TYPE_MASK) == VI_TYPE_8888;
		bool fetch_aa = (r.status & VI_META_AA) != 0;
		bool dither_filter = (r.status & VI_DITHER_FILTER) != 0;

		Img vram, aa, dv;
		if (!degenerate)
		{
			const auto src = sources();
			const uint8_t *rdram = src.first, *hidden = src.second;
			// extract_vram.comp
			int ew = r.max_x + 2 + 4 + int(divot) * 2, eh = r.max_y + 1 + 4;
			vram.init(ew, eh, 1);
			int fb_offset = is_8888 ? (r.vi_offset >> 2) : (r.vi_offset >> 1);
			int xo = divot ? -3 : -2, yo = -2;
			for (int y = 0; y < eh; y++)
				for (int x = 0; x < ew; x++)
				{
					int cx = x + xo, cy = y + yo;
					// extract_vram.comp:58-67: the sample slice of an upscaled pixel.
					const int slice = ((cy & (S - 1)) << L) + (cx & (S - 1));
					cx >>= L;
					cy >>= L;
					uint32_t c[4];
					int lin = cy * r.vi_width + cx + fb_offset;
					if (is_8888)
					{
						lin &= int((rdram_size >> 2) - 1);
						lin += slice * int(rdram_size >> 2);
						const uint8_t *p = rdram + size_t(lin) * 4;
						uint32_t w = uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
						c[0] = (w >> 24) & 0xff; c[1] = (w >> 16) & 0xff; c[2] = (w >> 8) & 0xff; c[3] = (w >> 5) & 7;
					}
					else
					{
						lin &= int((rdram_size >> 1) - 1);
						lin += slice * int(rdram_size >> 1);
						const uint8_t *p = rdram + size_t(lin ^ 1) * 2;
						uint32_t w = uint32_t(p[0]) | (uint32_t(p[1]) << 8);
						uint32_t hw = hidden[lin];
						c[0] = (w >> 8) & 0xf8; c[1] = (w >> 3) & 0xf8; c[2] = (w << 2) & 0xf8; c[3] = ((w & 1) << 2) | hw;
					}
					if (!fetch_aa) c[3] = 7;
					uint8_t *d = vram.at(x, y, 0);
					for (int i = 0; i < 4; i++) d[i] = uint8_t(c[i]);
				}

			// vi_fetch.frag
			int aw = r.max_x + 3 + int(divot) * 2, ah = r.max_y + 2;
			aa.init(aw, ah, fetch_bug ? 2 : 1);
			for (int y = 0; y < ah; y++)
				for (int x = 0; x < aw; x++)
				{
					int px = x + 2, py = y + 2;
					uint32_t mid[4];
					vram.get(px, py, 0, mid);
					uint32_t col[3], bug[3];
					if (mid[3] != 7)
					{
						uint32_t lo[3], hi[3], slo[3], shi[3];
						for (int i = 0; i < 3; i++) lo[i] = hi[i] = slo[i] = shi[i] = mid[i];
						uint32_t n[6][4];
						vram.get(px - 1, py - 1, 0, n[0]);
						vram.get(px + 1, py - 1, 0, n[1]);
						vram.get(px - 2, py, 0, n[2]);
						vram.get(px + 2, py, 0, n[3]);
						vram.get(px - 1, py + 1, 0, n[4]);
						vram.get(px + 1, py + 1, 0, n[5]);
						auto check = [](const uint32_t *c, uint32_t *lo_, uint32_t *hi_, uint32_t *slo_, uint32_t *shi_) {
							if (c[3] == 7)
								for (int i = 0; i < 3; i++)
								{
									slo_[i] = std::min(slo_[i], std::max(c[i], lo_[i]));
									shi_[i] = std::max(shi_[i], std::min(c[i], hi_[i]));
									lo_[i] = std::min(c[i], lo_[i]);
									hi_[i] = std::max(c[i], hi_[i]);
								}
						};
						for (int k = 0; k < 4; k++) check(n[k], lo, hi, slo, shi);
						uint32_t lob[3], hib[3], slob[3], shib[3];
						memcpy(lob, lo, sizeof(lo)); memcpy(hib, hi, sizeof(hi));
						memcpy(slob, slo, sizeof(slo)); memcpy(shib, shi, sizeof(shi));
						check(n[4], lo, hi, slo, shi);
						check(n[5], lo, hi, slo, shi);
						if (fetch_bug)
						{
							check(n[2], lob, hib, slob, shib);
							check(n[3], lob, hib, slob, shib);
							for (int i = 0; i < 3; i++)
							{
								if (mid[i] == lo[i]) slo[i] = lo[i];
								if (mid[i] == hi[i]) shi[i] = hi[i];
								if (mid[i] == lob[i]) slob[i] = lob[i];
								if (mid[i] == hib[i]) shib[i] = hib[i];
							}
						}
						uint32_t coeff = 7u - mid[3];
						for (int i = 0; i < 3; i++)
						{
							uint32_t off = slo[i] + shi[i] - (mid[i] << 1);
							col[i] = (mid[i] + (((off * coeff) + 4u) >> 3)) & 0xff;
							uint32_t offb = slob[i] + shib[i] - (mid[i] << 1);
							bug[i] = (mid[i] + (((offb * coeff) + 4u) >> 3)) & 0xff;
						}
					}
					else if (dither_filter)
					{
						int tc[3], acc[3] = { 0, 0, 0 }, accb[3];
						for (int i = 0; i < 3; i++) tc[i] = int(mid[i] >> 3);
						auto add = [&](int dx, int dy, int *a) {
							uint32_t c[4];
							vram.get(px + dx, py + dy, 0, c);
							for (int i = 0; i < 3; i++) a[i] += std::min(std::max(int(c[i] >> 3) - tc[i], -1), 1);
						};
						for (int yy = -1; yy <= 0; yy++)
							for (int xx = -1; xx <= 1; xx++) add(xx, yy, acc);
						memcpy(accb, acc, sizeof(acc));
						add(-1, 1, acc);
						add(1, 1, acc);
						add(0, 1, acc);
						add(-1, 0, accb);
						add(1, 0, accb);
						for (int i = 0; i < 3; i++)
						{
							col[i] = uint32_t(int(mid[i] & 0xf8) + acc[i]);
							bug[i] = uint32_t(int(mid[i] & 0xf8) + accb[i]);
						}
					}
					else
						for (int i = 0; i < 3; i++) col[i] = bug[i] = mid[i];
					// The fetch image is an 8-bit unsigned integer target: values wrap to 8 bits.
					uint8_t *d = aa.at(x, y, 0);
					for (int i = 0; i < 3; i++) d[i] = uint8_t(col[i]);
					d[3] = uint8_t(mid[3]);
					if (fetch_bug)
					{
						uint8_t *e = aa.at(x, y, 1);
						for (int i = 0; i < 3; i++) e[i] = uint8_t(bug[i]);
						e[3] = uint8_t(mid[3]);
					}
				}

			if (divot)
			{
				// vi_divot.frag
				int dw = r.max_x + 2, dh = r.max_y + 2;
				dv.init(dw, dh, aa.layers);
				for (int l = 0; l < aa.layers; l++)
					for (int y = 0; y < dh; y++)
						for (int x = 0; x < dw; x++)
						{
							uint32_t le[4], mi[4], ri[4];
							aa.get(x, y, l, le);
							aa.get(x + 1, y, l, mi);
							aa.get(x + 2, y, l, ri);
							uint8_t *d = dv.at(x, y, l);
							if ((le[3] & mi[3] & ri[3]) == 7)
								for (int i = 0; i < 4; i++) d[i] = uint8_t(mi[i]);
							else
							{
								for (int i = 0; i < 3; i++)
								{
									uint32_t a = le[i], b = mi[i], c = ri[i];
									if (a < b) std::swap(a, b);
									if (b < c) std::swap(b, c);
									if (a < b) std::swap(a, b);
									d[i] = uint8_t(b);
								}
								d[3] = uint8_t(mi[3]);
							}
						}
			}
			else
				dv = aa;
		}

		// vi_scale.frag + blend of the previous frame (video_interface.cpp:719-988).
		bool serrate = (r.status & VI_SERRATE) != 0 && !o.upscale_deinterlacing;
		int width = SCANOUT_WIDTH * S, height = ((r.is_pal ? V_RES_PAL : V_RES_NTSC) >> int(!serrate)) * S;
		unsigned cl = 0, cr = 0, ct = 0, cb = 0;
		if (o.crop_rect_enable)
		{
			cl = o.crop_left; cr = o.crop_right; ct = o.crop_top; cb = o.crop_bottom;
			if (serrate) { ct *= 2; cb *= 2; }
		}
		else
		{
			unsigned cy = o.crop_overscan_pixels * (serrate ? 2 : 1);
			unsigned cx = unsigned(std::round(float(cy) * (float(width) / float(height))));
			cl = cr = cx;
			ct = cb = cy;
		}
		cl *= unsigned(S);
		cr *= unsigned(S);
		ct *= unsigned(S);
		cb *= unsigned(S);
		if (cl + cr < unsigned(width) && ct + cb < unsigned(height))
		{
			width -= int(cl + cr);
			height -= int(ct + cb);
		}
		out.init(width, height, 1);

		int v_start = r.v_start, v_res = r.v_res;
		int serrate_shift = 0, serrate_mask = 0, serrate_select = 0, info_y_shift = L;
		if (serrate)
		{
			v_start *= 2;
			v_res *= 2;
			serrate_shift = 1;
			serrate_mask = 1;
			serrate_select = int(r.v_current_line == 0);
			info_y_shift++;
		}
		bool scale_aa = (r.status & VI_META_SCALE) != 0;
		bool gamma_en = (r.status & VI_GAMMA) != 0, gamma_dither = (r.status & VI_GAMMA_DITHER) != 0;

		auto in_rect = [](int x, int y, int rx, int ry, int rw, int rh, int crop_x, int crop_y) {
			rx -= crop_x;
			ry -= crop_y;
			if (rx < 0) { rw += rx; rx = 0; }
			if (ry < 0) { rh += ry; ry = 0; }
			if (rw <= 0 || rh <= 0) return false;
			return x >= rx && x < rx + rw && y >= ry && y < ry + rh;
		};

		if (!degenerate && r.h_res > 0 && r.v_res > 0)
		{
			for (int fy = 0; fy < height; fy++)
				for (int fx = 0; fx < width; fx++)
				{
					if (!in_rect(fx, fy, r.h_start, v_start, r.h_res, v_res, int(cl), int(ct))) continue;
					int cxp = fx + int(cl), cyp = fy + int(ct);
					const Line &li = lines[std::min(cyp >> info_y_shift, MAX_OUTPUT_SCANLINES - 1)];
					cyp -= v_start;
					if (cxp < li.h_start_clamp || cxp >= li.h_end_clamp || ((cyp & serrate_mask) != serrate_select))
						continue;
					cxp -= li.h_start;
					cyp >>= serrate_shift;
					uint32_t seed = 0;
					if (gamma_dither)
					{
						const uint32_t P = 1103515245u;
						uint32_t s0 = uint32_t(cxp), s1 = uint32_t(cyp), s2 = frame_count;
						for (int k = 0; k < 3; k++)
						{
							uint32_t n0 = ((s0 >> 8) ^ s1) * P, n1 = ((s1 >> 8) ^ s2) * P, n2 = ((s2 >> 8) ^ s0) * P;
							s0 = n0; s1 = n1; s2 = n2;
						}
						seed = (s0 >> 16) & 0xffff;
					}
					int x = cxp * li.x_add + li.x_start;
					int y = (cyp - li.y_base) * li.y_add + li.y_start;
					int bx = x >> 10, by = y >> 10;
					uint32_t c00[4];
					dv.get(bx, by, 0, c00);
					int bug_offset = 0;
					if (fetch_bug)
					{
						int prev_y = (y - r.init_y_add) >> 10, next_y = (y + r.init_y_add) >> 10;
						if (cyp != 0 && by == prev_y && by != next_y) bug_offset = 1;
					}
					uint32_t res[3] = { c00[0], c00[1], c00[2] };
					if (scale_aa)
					{
						uint32_t xf = uint32_t((x >> 5) & 31), yf = uint32_t((y >> 5) & 31);
						uint32_t c10[4], c01[4], c11[4];
						dv.get(bx + 1, by, 0, c10);
						dv.get(bx, by + 1, bug_offset, c01);
						dv.get(bx + 1, by + 1, bug_offset, c11);
						for (int i = 0; i < 3; i++)
						{
							uint32_t a = (c00[i] + (((c01[i] - c00[i]) * yf + 16u) >> 5)) & 0xff;
							uint32_t b = (c10[i] + (((c11[i] - c10[i]) * yf + 16u) >> 5)) & 0xff;
							res[i] = (a + (((b - a) * xf + 16u) >> 5)) & 0xff;
						}
					}
					if (gamma_en)
					{
						for (int i = 0; i < 3; i++)
						{
							uint32_t idx = res[i];
							if (gamma_dither)
							{
								uint32_t d = i == 0 ? (seed & 0x3f) : i == 1 ? ((seed >> 6) & 0x3f) : (((seed >> 9) & 0x38) | (seed & 7));
								idx = (res[i] << 6) + d + 256u;
							}
							res[i] = gamma[std::min<uint32_t>(idx, 256 + 256 * 64 - 1)];
						}
					}
					else if (gamma_dither)
						for (int i = 0; i < 3; i++) res[i] = std::min<uint32_t>(res[i] + ((seed >> i) & 1u), 0xff);
					uint8_t *d = out.at(fx, fy, 0);
					d[0] = uint8_t(res[0]); d[1] = uint8_t(res[1]); d[2] = uint8_t(res[2]); d[3] = 255;
				}
		}

		if (have_prev && o.blend_previous_frame)
		{
			auto blend = [&](int rx, int ry, int rw, int rh) {
				for (int fy = 0; fy < height; fy++)
					for (int fx = 0; fx < width; fx++)
					{
						if (!in_rect(fx, fy, rx, ry, rw, rh, int(cl), int(ct))) continue;
						uint8_t *d = out.at(fx, fy, 0);
						if (d[3] == 255) continue; // destination alpha 1 keeps the new pixel
						uint32_t p[4];
						prev.get(fx, fy, 0, p);
						for (int i = 0; i < 3; i++) d[i] = p[3] == 255 ? uint8_t(p[i]) : 0;
					}
			};
			if (degenerate)
			{
				if (r.h_res > 0) blend(r.h_start, 0, r.h_res, prev.h);
			}
			else
			{
				if (r.h_res > 0 && v_start > 0) blend(r.h_start, 0, r.h_res, v_start);
				if (r.h_res_clamp > 0 && v_res > 0) blend(r.h_start_clamp, v_start, r.h_res_clamp, v_res);
				if (r.h_res > 0 && prev.h > v_start + v_res) blend(r.h_start, v_start + v_res, r.h_res, prev.h - (v_start + v_res));
			}
		}
		// downscale_stage (video_interface.cpp:1000-1064): each step halves the image; the
		// reference's linear blit of exactly 2:1 is the mean of each 2x2 block, rounded half up.
		for (int steps = int(std::min(8u, o.downscale_steps)), f = S; f > 1 && steps > 0; f >>= 1, steps--)
		{
			Img half;
			half.init(out.w / 2, out.h / 2, 1);
			for (int y = 0; y < half.h; y++)
				for (int x = 0; x < half.w; x++)
				{
					uint32_t a[4], b[4], c[4], d[4];
					out.get(2 * x, 2 * y, 0, a);
					out.get(2 * x + 1, 2 * y, 0, b);
					out.get(2 * x, 2 * y + 1, 0, c);
					out.get(2 * x + 1, 2 * y + 1, 0, d);
					uint8_t *q = half.at(x, y, 0);
					for (int i = 0; i < 4; i++) q[i] = uint8_t((a[i] + b[i] + c[i] + d[i] + 2) >> 2);
				}
			out = half;
		}
		prev = out;
		have_prev = true;
		frame_count++;
		return true;
	}

	// video_interface.cpp:1102-1213
	void begin_per_scanline(uint32_t flags)
	{
		ps_flags = flags;
		hs_latched = regs[9];
		xs_latched = regs[12];
		hs_line[0] = regs[9];
		xs_line[0] = regs[12];
		ps_line = 0;
		ps_ended = false;
	}
	void set_for_scanline(uint32_t reg, uint32_t value)
	{
		if ((ps_flags & reg) == 0) return;
		if (reg == 1) hs_latched = value;
		else if (reg == 2) xs_latched = value;
	}
	void latch_scanline(unsigned line)
	{
		line = std::min<unsigned>(line, V_END_MAX - 1);
		if (line <= ps_line) return;
		unsigned c = ps_line;
		while (++c < line)
		{
			hs_line[c] = hs_line[ps_line];
			xs_line[c] = xs_line[ps_line];
		}
		hs_line[c] = hs_latched;
		xs_line[c] = xs_latched;
		ps_line = c;
	}
	void end_per_scanline()
	{
		if (ps_flags == 0 || ps_ended) return;
		unsigned c = ps_line;
		while (++c < unsigned(V_END_MAX))
		{
			hs_line[c] = hs_line[ps_line];
			xs_line[c] = xs_line[ps_line];
		}
		ps_ended = true;
	}
};

// Accessors into the renderer oracle (rdp_oracle.cpp).
extern "C" void oracle_read_rdram(void *h, uint8_t *data, uint32_t offset, uint32_t size);
extern "C" void oracle_read_hidden(void *h, uint8_t *data, uint32_t offset, uint32_t size);
extern "C" uint32_t oracle_rdram_size(void *h);
extern "C" uint32_t oracle_hidden_size(void *h);
extern "C" void *oracle_vi_state(void *h);
extern "C" void oracle_set_vi_state(void *h, void *vi);
extern "C" uint32_t oracle_upscaling_factor(void *h);
extern "C" void oracle_read_upscaled_rdram(void *h, uint8_t *data, uint64_t offset, uint64_t size);
extern "C" void oracle_read_upscaled_hidden(void *h, uint8_t *data, uint64_t offset, uint64_t size);
extern "C" void oracle_upscale_pre_external(void *h, uint32_t offset, uint32_t length, uint32_t psl2);

static ViOracle *vi_of(void *h)
{
	ViOracle *v = static_cast<ViOracle *>(oracle_vi_state(h));
	if (!v)
	{
		v = new ViOracle();
		oracle_set_vi_state(h, v);
	}
	return v;
}

extern "C" {

void oracle_vi_destroy(void *vi) { delete static_cast<ViOracle *>(vi); }

void oracle_set_vi_register(void *h, uint32_t reg, uint32_t value)
{
	if (reg < 14) vi_of(h)->regs[reg] = value;
}
void oracle_vi_begin_per_scanline(void *h, uint32_t flags) { vi_of(h)->begin_per_scanline(flags); }
void oracle_vi_set_for_scanline(void *h, uint32_t reg, uint32_t value) { vi_of(h)->set_for_scanline(reg, value); }
void oracle_vi_latch_scanline(void *h, uint32_t line) { vi_of(h)->latch_scanline(line); }
void oracle_vi_end_per_scanline(void *h) { vi_of(h)->end_per_scanline(); }

// opts: 16 uint32 in ViOracle::Options order.  out: capacity (640 x 576) x factor^2 RGBA8 words.
int oracle_scanout(void *h, const uint32_t *opts, uint32_t *out, uint32_t *width, uint32_t *height)
{
	ViOracle *v = vi_of(h);
	ViOracle::Options o;
	memcpy(&o, opts, sizeof(o));
	uint32_t rs = oracle_rdram_size(h), hs = oracle_hidden_size(h);
	const uint32_t factor = oracle_upscaling_factor(h);
	const uint32_t raw_status = v->regs[0];
	std::vector<uint8_t> rd, hid;
	auto sources = [&]() -> std::pair<const uint8_t *, const uint8_t *> {
		if (factor > 1)
		{
			// The fetch first brings the scanned range of the upscaled domain up to date with RDRAM
			// (VideoInterface::vram_fetch_stage, video_interface.cpp:410-420); the pixel size follows
			// the status with the RGBA5551 bit forced (video_interface.cpp:1256).
			uint32_t offset, length;
			v->memory_range(offset, length);
			uint32_t psl2 = ((raw_status & VI_TYPE_MASK) | VI_TYPE_5551) == VI_TYPE_8888 ? 2 : 1;
			oracle_upscale_pre_external(h, offset, length, psl2);
			rd.resize(size_t(rs) * factor * factor);
			hid.resize(size_t(hs) * factor * factor);
			oracle_read_upscaled_rdram(h, rd.data(), 0, rd.size());
			oracle_read_upscaled_hidden(h, hid.data(), 0, hid.size());
		}
		else
		{
			rd.resize(rs);
			hid.resize(hs);
			oracle_read_rdram(h, rd.data(), 0, rs);
			oracle_read_hidden(h, hid.data(), 0, hs);
		}
		return { rd.data(), hid.data() };
	};
	Img img;
	if (!v->scanout(o, sources, rs, img, int(factor)))
	{
		*width = *height = 0;
		return 0;
	}
	*width = uint32_t(img.w);
	*height = uint32_t(img.h);
	for (int i = 0; i < img.w * img.h; i++)
		out[i] = uint32_t(img.px[i * 4]) | (uint32_t(img.px[i * 4 + 1]) << 8) | (uint32_t(img.px[i * 4 + 2]) << 16) |
		         (uint32_t(img.px[i * 4 + 3]) << 24);
	return 1;
}
}
