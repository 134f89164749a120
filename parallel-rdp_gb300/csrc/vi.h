/*
 * Video Interface (scanout) of the GB300 RDP path: parameters shared by the host
 * (rdp_cp.cpp, register decode and frame logic of video_interface.cpp:177-1426)
 * and the kernels (vi.cu: extract_vram.comp + vi_fetch.frag, vi_divot.frag,
 * vi_scale.frag + vi_blend_fields.frag as CUDA kernels).
 */
#ifndef RDP_VI_H
#define RDP_VI_H

#include <cuda_runtime.h>
#include <stdint.h>

#define RDP_VI_MAX_LINES 288

typedef struct RdpViLine
{
	int32_t h_start, h_start_clamp, h_end_clamp, x_start, x_add, y_start, y_add, y_base;
} RdpViLine;

typedef struct RdpViParams
{
	// Sources.
	const uint8_t *rdram;
	const uint8_t *hidden;
	uint32_t rdram_size;
	int32_t fb_offset;    // in pixels of the VI format
	int32_t fb_width;
	int32_t is_8888;
	int32_t fetch_aa;     // coverage from memory, else 7
	int32_t dither_filter;
	int32_t divot;
	int32_t fetch_bug;
	int32_t degenerate;
	// Intermediate images (RGBA8, [layer][h][w]).
	uint32_t *aa;
	int32_t aa_w, aa_h;
	uint32_t *dv;
	int32_t dv_w, dv_h;
	// Scale pass.
	const RdpViLine *lines;
	uint32_t *out;
	int32_t out_w, out_h;
	const uint32_t *prev;
	int32_t prev_w, prev_h;
	int32_t crop_left, crop_top;
	int32_t v_start, v_res, h_start, h_res, h_start_clamp, h_res_clamp;
	int32_t draw; // the scale pass draws
	int32_t serrate_shift, serrate_mask, serrate_select, info_y_shift;
	int32_t init_y_add;
	uint32_t frame_count;
	int32_t scale_aa, gamma, gamma_dither;
	int32_t blend_prev;
	// Upscaling: log2 of the factor.  rdram / hidden are then the multisampled copies (factor^2
	// slices of rdram_size / rdram_size / 2 bytes) and the images are in scaled pixels.
	int32_t scale_log2;
} RdpViParams;

#ifdef __cplusplus
extern "C" {
#endif
cudaError_t rdp_vi_init_tables(void);
cudaError_t rdp_vi_launch(const RdpViParams *p, cudaStream_t stream);
/* One step of downscale_stage (video_interface.cpp:1000-1064): dst (w / 2 x h / 2) = the 2x2 means
 * of src (w x h), rounded half up. */
cudaError_t rdp_vi_downscale(const uint32_t *src, int32_t w, int32_t h, uint32_t *dst, cudaStream_t stream);
#ifdef __cplusplus
}
#endif
#endif
