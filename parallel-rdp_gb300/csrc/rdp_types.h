/*
 * Host/device data layouts of the GB300 RDP path.
 *
 * The host command processor (rdp_cp.cpp) does a light, sequential parse of the
 * RDP command stream: it tracks the state registers as raw command words
 * ("state blocks"), decodes tile descriptors and plans TMEM uploads (these are
 * inherently sequential), and records one 16-byte PrimIn per drawn primitive.
 * All per-primitive decoding -- edge/attribute coefficients, derived combiner
 * constants, state normalisation -- runs on the GPU (k_prim_setup), followed by
 * binning (k_bin), TMEM snapshot generation (k_tmem) and the fused per-tile
 * rasteriser (k_raster).
 *
 * A "pass" is a run of primitives that share one colour/depth image and may be
 * rendered concurrently tile-by-tile (the reference's render pass,
 * rdp_renderer.cpp:2909-2986, with larger limits).  A launch renders one or
 * more passes, each belonging to an emulator instance with its own RDRAM.
 */
#ifndef RDP_TYPES_H
#define RDP_TYPES_H

#include <stdint.h>

#define RDP_TILE_W 8
#define RDP_TILE_H 8
#define RDP_MAX_PRIMS_PER_PASS 65536
#define RDP_MAX_UPLOADS_PER_PASS 16384
/* 32-bit words of one tile's primitive bitmask for a pass of `prims` primitives: one bit per
 * primitive, padded to whole 16-byte groups (k_expand reads a bitmask four words at a time). */
#define RDP_MASK_WORDS(prims) ((((prims) + 127u) >> 7) << 2)
#define RDP_MAX_TILES_X 128
#define RDP_MAX_TILES_Y 128
#define RDP_STATE_BLOCK_WORDS 32

/* Indices of raw state words inside a state block. */
enum
{
	SB_OTHER_MODES = 0,
	SB_COMBINE = 2,
	SB_SCISSOR = 4,
	SB_PRIM_COLOR = 6,
	SB_ENV_COLOR = 8,
	SB_BLEND_COLOR = 10,
	SB_FOG_COLOR = 12,
	SB_FILL_COLOR = 14,
	SB_CONVERT = 16,
	SB_KEY_R = 18,
	SB_KEY_GB = 20,
	SB_PRIM_DEPTH = 22,
	SB_QUIRKS = 24
};

/* Flag bit values follow the reference's enums (rdp_data_structures.hpp:31-93). */
enum
{
	TRI_FLIP = 1 << 0,
	TRI_DO_OFFSET = 1 << 1,
	TRI_SKIP_XFRAC = 1 << 2,
	TRI_INTERLACE_FIELD = 1 << 3,
	TRI_INTERLACE_KEEP_ODD = 1 << 4,
	TRI_DISABLE_UPSCALING = 1 << 5,
	TRI_NATIVE_LOD = 1 << 6,
	TRI_FILL_COPY_RASTER = 1 << 7
};

enum
{
	RS_INTERLACE_FIELD = 1u << 0,
	RS_INTERLACE_KEEP_ODD = 1u << 1,
	RS_AA = 1u << 2,
	RS_PERSPECTIVE = 1u << 3,
	RS_TLUT = 1u << 4,
	RS_TLUT_TYPE = 1u << 5,
	RS_CVG_TIMES_ALPHA = 1u << 6,
	RS_ALPHA_CVG_SELECT = 1u << 7,
	RS_MULTI_CYCLE = 1u << 8,
	RS_TEX_LOD = 1u << 9,
	RS_SHARPEN = 1u << 10,
	RS_DETAIL = 1u << 11,
	RS_FILL = 1u << 12,
	RS_COPY = 1u << 13,
	RS_SAMPLE_QUAD = 1u << 14,
	RS_ALPHA_TEST = 1u << 15,
	RS_ALPHA_TEST_DITHER = 1u << 16,
	RS_MID_TEXEL = 1u << 17,
	RS_USES_TEXEL0 = 1u << 18,
	RS_USES_TEXEL1 = 1u << 19,
	RS_USES_LOD = 1u << 20,
	RS_USES_PIPELINED_TEXEL1 = 1u << 21,
	RS_CONVERT_ONE = 1u << 22,
	RS_BILERP0 = 1u << 23,
	RS_BILERP1 = 1u << 24,
	RS_NEED_NOISE_DUAL = 1u << 25,
	RS_NEED_NOISE = 1u << 28
};

enum
{
	DB_DEPTH_TEST = 1u << 0,
	DB_DEPTH_UPDATE = 1u << 1,
	DB_FORCE_BLEND = 1u << 3,
	DB_IMAGE_READ = 1u << 4,
	DB_COLOR_ON_CVG = 1u << 5,
	DB_MULTI_CYCLE = 1u << 6,
	DB_AA = 1u << 7,
	DB_DITHER = 1u << 8
};

enum
{
	FBF_I4 = 0,
	FBF_I8 = 1,
	FBF_RGBA5551 = 2,
	FBF_IA88 = 3,
	FBF_RGBA8888 = 4
};

enum
{
	TIF_CLAMP_S = 1,
	TIF_MIRROR_S = 2,
	TIF_CLAMP_T = 4,
	TIF_MIRROR_T = 8
};

/* Decoded tile descriptor (rdp_common.hpp:255-322). */
typedef struct RdpTile
{
	uint32_t slo, shi, tlo, thi;
	uint32_t offset, stride;
	uint8_t fmt, size, palette, mask_s, shift_s, mask_t, shift_t, flags;
} RdpTile;

/* TMEM upload plan (rdp_data_structures.hpp:182-202). */
typedef struct RdpUpload
{
	int32_t width, height;
	float min_t_mod, max_t_mod;
	int32_t vram_addr, vram_width, vram_size, vram_effective_width;
	int32_t tmem_offset, tmem_stride_words, tmem_size, tmem_fmt;
	int32_t mode;
	float inv_tmem_stride_words;
	int32_t dxt;
	int32_t padding;
} RdpUpload;

/* One drawn primitive, as recorded by the host parser. */
typedef struct RdpPrimIn
{
	uint32_t word_offset;  /* first command word, in the launch's word buffer */
	uint32_t state_block;  /* index of the raw state-register block */
	uint32_t tileset;      /* index of the 8-tile descriptor set */
	uint16_t tmem_index;   /* TMEM snapshot the primitive samples (uploads before it in its pass) */
	uint16_t seq;          /* position of the primitive in its instance's pass, in command order */
} RdpPrimIn;

/* Per-primitive device records produced by k_prim_setup. */
typedef struct __attribute__((aligned(16))) RdpPrimGeom
{
	int32_t xh, xm, xl;
	int32_t yh, ym, yl;
	int32_t dxhdy, dxmdy, dxldy;
	uint32_t flags;     /* TRI_* */
	uint32_t tile;      /* tile | (max level << 3) */
	int32_t span_ylo, span_yhi;
	int32_t scissor[4]; /* xlo, ylo, xhi, yhi */
	uint16_t bbox[4];   /* conservative tile range: tx0, ty0, tx1, ty1 (tx1 < tx0 => none) */
	uint32_t pad[1];
} RdpPrimGeom;

typedef struct __attribute__((aligned(16))) RdpPrimAttr
{
	int32_t rgba[4], drgba_dx[4], drgba_de[4], drgba_dy[4];
	int32_t stzw[4], dstzw_dx[4], dstzw_de[4], dstzw_dy[4]; /* s, t, z, w */
} RdpPrimAttr;

typedef struct __attribute__((aligned(16))) RdpPrimShade
{
	uint32_t static_flags; /* normalised RS_* */
	uint32_t dither;       /* rgb mode << 2 | alpha mode */
	uint8_t comb_rgb[2][4];   /* normalised selectors: muladd, mulsub, mul, add */
	uint8_t comb_alpha[2][4];
	uint32_t db_flags;
	uint8_t blend[2][4];   /* 1a, 1b, 2a, 2b per cycle */
	uint8_t coverage_mode, z_mode, dz_compressed, min_lod;
	uint16_t dz;
	uint16_t tmem_index;
	uint8_t c_muladd[2][4], c_mulsub[2][4], c_mul[2][4], c_add[2][4];
	uint8_t fog[4], blend_color[4];
	uint32_t fill_color;
	int16_t factors[4];
	uint32_t tileset;
	uint32_t prim_index; /* global primitive index used to seed noise */
	uint32_t pass;
	uint32_t pad[3];
} RdpPrimShade;

/* Per-pass descriptor, device visible. */
typedef struct __attribute__((aligned(16))) RdpPass
{
	uint8_t *rdram;
	uint8_t *hidden;
	uint32_t *masks;    /* [tiles][mask_words]: bit p of a tile's words = primitive p of the pass binned there */
	uint16_t *tmem_snapshots; /* [uploads + 1][2048] */
	uint16_t *tmem_state;     /* the instance's persistent TMEM */
	uint32_t rdram_size, hidden_size;
	uint32_t fb_addr, depth_addr, fb_width, fb_height, fb_fmt;
	uint32_t tiles_x, tiles_y;
	uint32_t prim_begin, prim_count;
	uint32_t upload_begin, upload_count;
	uint32_t tile_item_begin; /* prefix over passes of tiles_x * tiles_y */
	uint32_t instance;
	uint32_t base_prim_index; /* primitives drawn by this instance before the pass (noise seed base) */
	/* Offsets of the pass's command words, state blocks and tile sets in the launch's buffers
	   (a primitive's word_offset / state_block / tileset are relative to its pass). */
	uint32_t word_base, sb_base, ts_base;
	/* Upscaled pass (the reference's render_pass_upscaled): bits 0-1 are log2 of the factor (0 for
	   a 1x pass); rdram / hidden are then the multisampled copies (factor^2 slices of rdram_size /
	   hidden_size bytes), fb_width / fb_height the scaled image.  Bit 8: record the super-sampled
	   write mask (2 bits per native pixel, after the slices). */
	uint32_t scale;
	uint32_t mask_words; /* 32-bit words of a tile's primitive bitmask: RDP_MASK_WORDS(prim_count) */
	unsigned long long *counters; /* the instance's [0] fragments, [1] touched tiles, [2] tile instances */
	uint32_t *wmask;              /* the instance's RDRAM write mask (1 bit per byte), or null */
} RdpPass;

/* RDRAM coherency with the caller's host memory (the reference's incoherent path,
 * rdp_renderer.cpp:2523-2907): pages of RDRAM_PAGE_BYTES. */
#define RDP_RDRAM_PAGE_BYTES 4096u


#endif
