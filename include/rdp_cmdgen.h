/*
 * Seeded synthetic RDP command-stream generator (input synthesis for tests and
 * benchmarks).  Plays the role of the reference's CommandBuilder
 * (rdp_command_builder.hpp:31-151) and triangle converter
 * (triangle_converter.cpp:129-273): random primitives in, raw RDP words out.
 */
#ifndef RDP_CMDGEN_H
#define RDP_CMDGEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum
{
	RDPGEN_FB_RGBA5551 = 0,
	RDPGEN_FB_RGBA8888 = 1,
	RDPGEN_FB_I8 = 2,
	RDPGEN_FB_IA88 = 3,
	RDPGEN_FB_I4 = 4
};

enum
{
	RDPGEN_CLEAR = 1u << 0,            /* FillRect clear of colour (and depth) at frame start */
	RDPGEN_Z = 1u << 1,                /* Z compare + update on every primitive */
	RDPGEN_2CYCLE = 1u << 2,           /* 2-cycle mode */
	RDPGEN_PERSPECTIVE = 1u << 3,      /* perspective-correct texturing */
	RDPGEN_BILINEAR = 1u << 4,         /* bilinear (sample quad) filtering */
	RDPGEN_AA = 1u << 5,               /* coverage AA */
	RDPGEN_DITHER = 1u << 6,           /* magic-square RGB dither */
	RDPGEN_FOG = 1u << 7,              /* fog blender */
	RDPGEN_RANDOM_COMBINER = 1u << 8,  /* combiner inputs drawn per primitive */
	RDPGEN_Z_HALF = 1u << 9,           /* Z on half of the primitives */
	RDPGEN_ALPHA_TEST_HALF = 1u << 10, /* alpha compare on half of the primitives */
	RDPGEN_LOD = 1u << 11,             /* random LOD / detail tiles on textured triangles */
	RDPGEN_RUNS = 1u << 12,            /* primitives of one kind come in runs */
	RDPGEN_FUZZ = 1u << 13,            /* every mode bit, selector, texture format and load drawn at random */
	RDPGEN_HOTSPOT = 1u << 14          /* triangle centroids inside the top-left 16x16 pixels (a few very busy tiles) */
};

typedef struct rdpgen_params
{
	uint32_t seed;
	uint32_t width, height;
	uint32_t fb_format;     /* RDPGEN_FB_* */
	uint32_t num_prims;     /* per frame */
	uint32_t num_frames;    /* each frame ends with SyncFull */
	float area_median;      /* pixels */
	float area_sigma;       /* log-normal sigma */
	uint32_t w_shade_tri, w_tex_tri, w_copy_rect, w_ci8_tri, w_fill_rect; /* mix weights */
	uint32_t flags;
	uint32_t rdram_size;
} rdpgen_params;

/* config: 0 = plain single frame, 1 = textured depth-tested frame, 2 = mixed 640x480 sequence. */
void rdpgen_default_params(rdpgen_params *p, int config);
void *rdpgen_build(const rdpgen_params *p);
void rdpgen_destroy(void *g);
uint32_t rdpgen_num_words(void *g);
const uint32_t *rdpgen_words(void *g);
uint32_t rdpgen_num_prims(void *g);
/* Frames of the stream and the word index where frame `frame` begins (num_words past the last). */
uint32_t rdpgen_num_frames(void *g);
uint32_t rdpgen_frame_word_offset(void *g, uint32_t frame);
/* Writes the generated texture/TLUT data into an RDRAM image (host-order words). */
void rdpgen_init_rdram(void *g, uint8_t *rdram, uint32_t size);
uint32_t rdpgen_color_addr(void);
uint32_t rdpgen_depth_addr(void);

#ifdef __cplusplus
}
#endif
#endif
