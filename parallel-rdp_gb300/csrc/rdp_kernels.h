/* Launch interface of the RDP kernels (rdp_kernels.cu). */
#ifndef RDP_KERNELS_H
#define RDP_KERNELS_H

#include <cuda_runtime.h>
#include "rdp_types.h"

/* Shading kernel variants (the autotuner chooses among them): k_shade_packedn<NP, R, SPEC> takes NP
 * (primitive, tile) pairs per warp step (their candidate pixels packed together) at a register
 * budget for R resident 64-thread CTAs per SM: the general shading code as <2, 18>, <3, 16>,
 * <4, 16>, <4, 18> (variants 0-3), separate code per render-state class as <2, 16 / 18 / 20 / 24>
 * (variants 4-7). */
/* Bytes of one span row (one scanline of one primitive, computed by k_bin). */
#define RDP_SPAN_ROW_BYTES 64
/* Launches with more tiles (or, in primitive-major order, primitives) than this scan their
 * pair counts with several CTAs. */
#define RDP_SCAN_SINGLE_CTA_MAX 16384

#ifndef RDP_SHADE_VARIANTS
#define RDP_SHADE_VARIANTS 8
#endif

typedef struct RdpLaunch
{
	const RdpPrimIn *prims_in;
	uint32_t num_prims;
	const uint32_t *words;
	const uint32_t *state_blocks;
	const RdpPass *passes;
	uint32_t num_passes;
	RdpPrimGeom *geom;
	RdpPrimAttr *attr;
	RdpPrimShade *shade;
	const RdpTile *tilesets;
	const uint32_t *tmem_pass_list;  /* descriptors of the passes with uploads, in launch order */
	const uint32_t *tmem_carry_list; /* the same, most uploads first (k_tmem_carry's grid order) */
	uint32_t num_tmem_passes;
	const RdpUpload *uploads;
	uint32_t num_uploads;     /* uploads of the launch (all TMEM passes' uploads, concatenated) */
	uint32_t *tmem_keep;      /* [num_uploads][64] scratch bitmask */
	uint32_t num_tile_items;
	cudaEvent_t shade_events[2];    /* optional: recorded around the k_shade launch */
	cudaEvent_t blend_events[2];    /* optional: recorded around the k_blend launch */
	const uint32_t *tile_order;     /* optional [num_tile_items]: order in which k_blend starts tiles */
	uint32_t *tile_cycles;          /* optional [num_tile_items]: measured k_blend cycles per tile */
	/* pair list + shading scratch */
	uint32_t *tile_counts;          /* [num_tile_items], zero between launches */
	uint32_t *nonempty_tiles;       /* [num_tile_items]: tiles with pairs, in tile order (k_scan) */
	uint32_t *scan_blocks;          /* [2 * ceil(num_tile_items / 1024)]: multi-CTA scan partials */
	uint32_t *pair_offsets;         /* [num_tile_items + 1] */
	uint2 *pairs;                   /* [pair_capacity] (global primitive index, tile item) */
	uint32_t *ctrl;                 /* [0] pairs, [1] overflow, [2] max pairs, [3] non-empty tiles, [4] counter,
	                                   [5] max span rows, [6..7] span-row counter, [8] device error word */
	uint32_t pair_capacity;
	uint32_t shade_ctas;            /* persistent CTAs of k_shade (and of k_blend / k_raster) */
	uint32_t *shade_queues;         /* optional [num_shade_queues + ceil(num_shade_queues / 32)]: per-SM
	                                   work queues of k_shade, then their used-up bitmask */
	uint32_t num_shade_queues;      /* the SM count */
	uint32_t shade_queue_min;       /* launches with fewer pairs per k_shade CTA take the fixed stride */
	uint4 *shade_list;              /* optional [pair_capacity]: primitive-major shading order, one
	                                   {primitive, tx | ty << 16, pair index, pass} record per position */
	uint32_t *prim_pairs;           /* [num_prims] pair count per primitive (with shade_list) */
	uint32_t *prim_offsets;         /* [num_prims] first primitive-major position (with shade_list) */
	uint32_t *prim_scan_blocks;     /* [2 * ceil(num_prims / 1024)] (with shade_list) */
	uint32_t shade_variant;         /* which compiled k_shade (register budget), < RDP_SHADE_VARIANTS */
	uint32_t blend_ctas;            /* persistent CTAs of k_blend / k_raster */
	uint32_t blend_kernel;          /* 0: k_blend_lookahead (inputs through registers), 1: k_blend (shared-memory
	                                   ring filled by bulk copies) */
	uint32_t *pair_log;             /* optional: k_scan writes the launch's pair count to pair_log[log_slot] */
	uint32_t log_slot;
	const struct RdpSchedDev *sched; /* optional learned tile order / online training (sched.h) */
	void *spans;                    /* [span_capacity] span rows (RDP_SPAN_ROW_BYTES each) */
	uint32_t span_capacity;
	uint32_t *prim_rows;            /* [num_prims] first span row of each primitive */
	uint32_t num_sms;               /* the device's SM count (sizes k_span's CTAs) */
	uint2 *scratch;                 /* [pair_capacity * 64] shaded records, 8 bytes per pixel */
	uint32_t upscaled;              /* the passes are upscaled passes (RdpPass.scale): set-up, binning, TMEM and
	                                   k_raster_upscaled only */
	uint32_t fill_only;             /* every primitive fills a rectangle: set-up, binning, TMEM and k_fill only */
	cudaStream_t side_stream;       /* optional: the TMEM kernels of a rasterising launch run here, forked
	                                   after fork_event and joined (join_event) before shading */
	cudaEvent_t fork_event, join_event;
} RdpLaunch;

#ifdef __cplusplus
extern "C" {
#endif
cudaError_t rdp_kernels_init_luts(const uint8_t *blender_lut);
cudaError_t rdp_kernels_launch(const RdpLaunch *launch, cudaStream_t stream);
uint32_t rdp_kernels_count(const RdpLaunch *launch);
int rdp_kernels_shade_ctas_per_sm(int variant);
int rdp_kernels_blend_ctas_per_sm(int kernel);
#ifdef __cplusplus
}
#endif
#endif
