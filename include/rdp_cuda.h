/*
 * librdp_cuda -- C ABI of the GB300-native N64 RDP rendering path.
 *
 * This is the drop-in boundary for the reference's RDP::CommandProcessor
 * (parallel-rdp/rdp_device.hpp:111-197).  Every entry point takes plain
 * pointers and sizes and returns an int status (RDP_OK or an RDP_ERR_* code);
 * no exception or C++ type crosses it.  Each function names the reference
 * interface it replaces.
 *
 * Threading: a processor is used from one emulator thread at a time.  By default
 * command words are decoded synchronously by the calling thread (the reference's
 * PARALLEL_RDP_SINGLE_THREADED_COMMAND mode, rdp_device.cpp:144-158); with
 * RDP_CREATE_COMMAND_THREAD they go through a 4096-word ring to a decoder thread
 * of the processor, as in the reference's default mode (command_ring.cpp:71-134).
 * GPU work is asynchronous and tracked by a monotonically increasing 64-bit
 * timeline.
 *
 * RDRAM ownership: the caller owns RDRAM (rdp_device.cpp:81-87).  The GPU
 * renders into a device copy (HBM) kept coherent with the caller's buffer page
 * by page, as the reference's incoherent-host path does
 * (rdp_renderer.cpp:2523-2907): the buffer is registered and mapped, every pass
 * first reads the pages it needs (texture sources, images) from it -- except
 * bytes the GPU wrote and has not yet returned -- and a timeline value writes
 * back exactly the bytes the GPU wrote, before it completes.  Pages are read when
 * the pass runs on the GPU, so the caller does not modify pages that unfinished
 * work reads.  Hidden RDRAM and TMEM are owned by the processor
 * (rdp_device.cpp:120-131).
 */
#ifndef RDP_CUDA_H
#define RDP_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum
{
	RDP_OK = 0,
	RDP_ERR_UNSUPPORTED = 1, /* no usable CUDA device, or an unsupported request */
	RDP_ERR_OOM = 2,         /* device or pinned-host allocation failed */
	RDP_ERR_TIMEOUT = 3,     /* a bounded wait expired */
	RDP_ERR_INVALID = 4,     /* bad argument */
	RDP_ERR_DEVICE = 5,      /* a CUDA call failed */
	RDP_ERR_TOO_LARGE = 6    /* a request exceeds a fixed capacity of an allocation-free entry point */
};

/* Validation errors reported through the callback (rdp_renderer.hpp:75-95). */
enum
{
	RDP_VALIDATION_FILL_4BPP = 0,
	RDP_VALIDATION_FILL_DEPTH_TEST = 1,
	RDP_VALIDATION_FILL_DEPTH_WRITE = 2,
	RDP_VALIDATION_FILL_IMAGE_READ = 3,
	RDP_VALIDATION_COPY_32BPP = 4,
	RDP_VALIDATION_LOAD_TILE_4BPP = 5,
	RDP_VALIDATION_MULTILINE_TLUT = 6
};

typedef struct rdp_cp rdp_cp;

typedef void (*rdp_validation_cb)(void *user, int error, const char *message);

/* Mirrors the CommandProcessor constructor arguments (rdp_device.hpp:113-115). */
typedef struct rdp_create_info
{
	void *rdram;              /* caller-owned RDRAM base (may be NULL: processor allocates a host mirror) */
	size_t rdram_offset;      /* byte offset of RDRAM inside `rdram` */
	size_t rdram_size;        /* power of two, e.g. 8 MiB */
	size_t hidden_rdram_size; /* power of two, normally rdram_size / 2 */
	uint32_t flags;           /* RDP_CREATE_* (batch instances: 0) */
	int device;               /* CUDA device ordinal */
} rdp_create_info;

/* Creation flags. */
enum
{
	/* Decode command words on a thread of the processor (the reference's command ring,
	 * command_ring.cpp:71-134; rdp_device.cpp:144-158).  rdp_cp_enqueue, rdp_cp_signal_timeline,
	 * rdp_cp_flush and rdp_cp_set_quirks push into a 4096-word ring (blocking while it is full) and
	 * return; timeline values travel in band (MetaSignalTimeline) and rdp_cp_wait_timeline may be
	 * called while the thread decodes.  Calls that read or write processor state directly (RDRAM
	 * and TMEM access, scanout, statistics) first wait until the ring is drained.  Not for batch
	 * instances or sync-point captures. */
	RDP_CREATE_COMMAND_THREAD = 1u << 0,
	/* Internal upscaling by 2, 4 or 8 (the reference's COMMAND_PROCESSOR_FLAG_UPSCALING_*_BIT,
	 * rdp_device.hpp:43-52, rdp_device.cpp:189-205; the largest factor given wins).  Every render
	 * pass into a 16/32-bit image at least 256 pixels wide is rendered a second time at the scaled
	 * resolution into a multisampled copy of RDRAM (factor^2 slices; pixel (x, y) of the scaled
	 * image is slice (y % f) * f + x % f at the address of native pixel (x / f, y / f)); RDRAM
	 * itself still receives the 1x rendering.  The multisampled copy follows CPU writes and other
	 * passes' output through the reference's "pre" / "post" updates, and scanout reads it: images
	 * are f times larger (ScanoutOptions.downscale_steps halves them).  hidden_rdram_size must be
	 * rdram_size / 2.  Not for batch instances or sync-point captures. */
	RDP_CREATE_UPSCALING_2X = 1u << 2,
	RDP_CREATE_UPSCALING_4X = 1u << 3,
	RDP_CREATE_UPSCALING_8X = 1u << 4,
	/* Super-sampled readback (COMMAND_PROCESSOR_FLAG_SUPER_SAMPLED_READ_BACK_BIT): every pass
	 * renders only at the scaled resolution and each native pixel a sample wrote is resolved into
	 * RDRAM (mean of the samples for colour, the first sample for depth); needs an upscaling flag. */
	RDP_CREATE_SUPER_SAMPLED_READ_BACK = 1u << 5,
	/* With super-sampled readback: RGBA5551 means are ordered-dithered (4x4 Bayer). */
	RDP_CREATE_SUPER_SAMPLED_DITHER = 1u << 6
};

/* CommandProcessor::CommandProcessor (rdp_device.cpp:44-162). */
int rdp_cp_create(const rdp_create_info *info, rdp_cp **out);
/* CommandProcessor::~CommandProcessor (rdp_device.cpp:225-233). */
void rdp_cp_destroy(rdp_cp *cp);
/* CommandProcessor::device_is_supported (rdp_device.cpp:164-167): 1 when a CUDA device is usable. */
int rdp_device_is_supported(int device);

/* CommandProcessor::enqueue_command (rdp_device.cpp:874-897).  Accepts any
 * number of whole or partial commands; a trailing partial command is kept until
 * the rest of its words arrive.  The in-band meta ops of the reference's command
 * stream (rdp_common.hpp:37-43; rdp_device.cpp:926-952) are decoded too:
 * MetaSignalTimeline (op 1, three words: the op word, then the 64-bit value, low
 * word first), MetaFlush (op 2, one word), MetaIdle (op 3, one word; a hint with
 * no effect here) and MetaSetQuirks (op 4, two words). */
int rdp_cp_enqueue(rdp_cp *cp, uint32_t num_words, const uint32_t *words);

/* CommandProcessor::signal_timeline (rdp_device.cpp:1053-1065). */
int rdp_cp_signal_timeline(rdp_cp *cp, uint64_t *value);
/* CommandProcessor::wait_for_timeline (rdp_device.cpp:1067-1080), bounded by timeout_ns. */
int rdp_cp_wait_timeline(rdp_cp *cp, uint64_t value, uint64_t timeout_ns);
/* CommandProcessor::flush (rdp_device.cpp:1045-1051). */
int rdp_cp_flush(rdp_cp *cp);
/* CommandProcessor::idle (rdp_device.cpp:1039-1043). */
int rdp_cp_idle(rdp_cp *cp);
/* CommandProcessor::begin_frame_context (rdp_device.cpp:169-174). */
int rdp_cp_begin_frame_context(rdp_cp *cp);
/* CommandProcessor::set_quirks (rdp_device.cpp:961-968): the Quirks word. */
int rdp_cp_set_quirks(rdp_cp *cp, uint32_t quirks);
/* CommandProcessor::set_validation_interface (rdp_device.cpp:230-233). */
int rdp_cp_set_validation_callback(rdp_cp *cp, rdp_validation_cb cb, void *user);

/* CommandProcessor::begin_read_rdram / end_write_rdram / begin_read_hidden_rdram /
 * end_write_hidden_rdram / get_rdram_size / get_hidden_rdram_size / get_tmem
 * (rdp_device.cpp:996-1037).  begin_read_rdram idles and returns the caller's buffer;
 * end_write_rdram makes the next pass refresh every RDRAM page (writes are also picked
 * up without it, page by page, when a pass reads them). */
void *rdp_cp_begin_read_rdram(rdp_cp *cp);
int rdp_cp_end_write_rdram(rdp_cp *cp);
void *rdp_cp_begin_read_hidden_rdram(rdp_cp *cp);
int rdp_cp_end_write_hidden_rdram(rdp_cp *cp);
size_t rdp_cp_get_rdram_size(rdp_cp *cp);
size_t rdp_cp_get_hidden_rdram_size(rdp_cp *cp);
int rdp_cp_get_tmem(rdp_cp *cp, uint16_t *out_2048_words);

/* Renderer::get_scaling_factor (rdp_renderer.cpp:2694-2697): 1, 2, 4 or 8. */
uint32_t rdp_cp_get_scaling_factor(rdp_cp *cp);
/* The multisampled copies of an upscaling processor (Renderer::get_upscaled_rdram_buffer /
 * get_upscaled_hidden_rdram_buffer, rdp_renderer.cpp:2699-2707): idles, then copies `size` bytes
 * from byte `offset` of the factor^2 slices of RDRAM (of hidden RDRAM).  RDP_ERR_INVALID without
 * upscaling or past the end. */
int rdp_cp_read_upscaled_rdram(rdp_cp *cp, void *dst, uint64_t offset, uint64_t size);
int rdp_cp_read_upscaled_hidden_rdram(rdp_cp *cp, void *dst, uint64_t offset, uint64_t size);

/* CommandProcessor::set_vi_register (rdp_device.cpp:970-975); reg is VIRegister (rdp_common.hpp:286-302). */
int rdp_cp_set_vi_register(rdp_cp *cp, uint32_t reg, uint32_t value);

/* ScanoutOptions (video_interface.hpp:31-81).  Crop pixels are native pixels (scaled with the
 * image on an upscaling processor). */
typedef struct rdp_scanout_options
{
	uint32_t crop_overscan_pixels;
	uint32_t crop_rect_enable, crop_left, crop_right, crop_top, crop_bottom;
	uint32_t persist_frame_on_invalid_input;
	uint32_t blend_previous_frame;
	uint32_t upscale_deinterlacing; /* 1 (default): serrate is not woven at 1x; 0: weave the fields */
	uint32_t vi_aa, vi_scale, vi_serrate, vi_dither_filter, vi_divot_filter, vi_gamma_dither;
	/* Halvings of an upscaled image before output (video_interface.hpp:51; at most 8, and none past
	 * 1x; video_interface.cpp:1000-1064, 1354).  Each halving averages 2x2 pixels, rounded half up
	 * (the reference's 2:1 linear blit). */
	uint32_t downscale_steps;
} rdp_scanout_options;
/* Fills the reference's defaults (every VI filter on, upscale deinterlacing on). */
void rdp_scanout_options_default(rdp_scanout_options *opts);

/* CommandProcessor::scanout_sync (rdp_device.cpp:1130-1182): renders everything
 * queued, runs the VI filters on the device and writes the RGBA8 image
 * (r | g << 8 | b << 16 | a << 24 per pixel) into `rgba_out`, which must hold
 * 640 x 576 pixels times the square of the scaling factor.  A width/height of 0 means
 * no image (blank or invalid VI state).  opts may be NULL for the defaults. */
int rdp_cp_scanout_sync(rdp_cp *cp, const rdp_scanout_options *opts, uint32_t *rgba_out, uint32_t *width,
                        uint32_t *height);
/* A scanned-out image in device memory: width x height RGBA8 pixels (r | g << 8 | b << 16 | a << 24),
 * rows of `width` pixels.  Owned by the processor. */
typedef struct rdp_vi_image
{
	const uint32_t *pixels; /* device pointer; NULL: no image (blank or invalid VI state) */
	uint32_t width, height;
} rdp_vi_image;
/* CommandProcessor::scanout (rdp_device.cpp:1082-1128): renders everything queued and runs the VI
 * filters on the device; the reference returns a Vulkan image, this returns the image in device
 * memory.  The VI work has finished when the call returns.  The image stays valid until the second
 * scanout after this one (two images alternate: the previous one is the source of the
 * previous-frame blend). */
int rdp_cp_scanout(rdp_cp *cp, const rdp_scanout_options *opts, rdp_vi_image *out);

/* VIScanoutBuffer (video_interface.hpp:83-89): a host copy of a scanout and the fence of that copy.
 * Zero-initialise before first use; the library (re)allocates `pixels` (pinned host memory) and
 * creates `fence`; rdp_vi_scanout_buffer_release frees both. */
typedef struct rdp_vi_scanout_buffer
{
	uint32_t *pixels;       /* width x height RGBA8 pixels once the fence has completed */
	size_t capacity_pixels;
	uint32_t width, height; /* 0 x 0: no image */
	void *fence;            /* the copy's completion event */
} rdp_vi_scanout_buffer;
/* CommandProcessor::scanout_async_buffer (rdp_device.cpp:1130-1158): queues the scanout and the copy
 * of the image into `buf` and returns without waiting for them. */
int rdp_cp_scanout_async_buffer(rdp_cp *cp, const rdp_scanout_options *opts, rdp_vi_scanout_buffer *buf);
/* Waits for the buffer's copy (the reference's buffer.fence->wait()), bounded by timeout_ns. */
int rdp_vi_scanout_buffer_wait(rdp_vi_scanout_buffer *buf, uint64_t timeout_ns);
void rdp_vi_scanout_buffer_release(rdp_vi_scanout_buffer *buf);

/* Per-scanline HStart/XScale (video_interface.hpp PerScanlineRegisterBits: 1 = HStart, 2 = XScale):
 * CommandProcessor::begin/set/latch/end_vi_register_per_scanline (rdp_device.cpp:977-995). */
int rdp_cp_begin_vi_register_per_scanline(rdp_cp *cp, uint32_t flags);
int rdp_cp_set_vi_register_for_scanline(rdp_cp *cp, uint32_t reg_bit, uint32_t value);
int rdp_cp_latch_vi_register_for_scanline(rdp_cp *cp, uint32_t vi_line);
int rdp_cp_end_vi_register_per_scanline(rdp_cp *cp);

/* Counters for benchmarking: primitives drawn, passes submitted, reference-equivalent
 * render passes (the reference's <=256-primitive segmentation, rdp_renderer.cpp:1564-1590),
 * fragments processed by the depth/blend, fill and copy pipes. */
typedef struct rdp_stats
{
	uint64_t primitives;
	uint64_t passes;
	uint64_t reference_passes;
	uint64_t fragments;
	uint64_t tmem_uploads;
	uint64_t touched_tiles;   /* 8x8 tiles the rasteriser loaded and stored */
	uint64_t kernel_launches; /* kernels this processor launched (graph replays included) */
	uint64_t staging_bytes;   /* host->device bytes of command/state data */
	uint64_t tile_instances;  /* (primitive, 8x8 tile) pairs shaded */
} rdp_stats;
int rdp_cp_get_stats(rdp_cp *cp, rdp_stats *out);

/* Sync-point capture (the reference submits each sync point's render passes as one
 * command buffer, rdp_renderer.cpp:2909-2986; here they become one CUDA graph).
 * Between rdp_cp_capture_begin and rdp_cp_capture_end, flushed passes are not run:
 * their command data is copied once into device memory and their kernels are
 * recorded.  rdp_graph_replay launches the recorded kernels `count` times on the
 * processor's stream, with every input already resident in HBM, and waits.  The framebuffer
 * ranges the recorded passes write are copied back to the caller's RDRAM with the processor's
 * next timeline value (as for passes run normally).  A graph is destroyed before its processor
 * (a batch's graph skips instances destroyed since the capture). */
typedef struct rdp_graph rdp_graph;
int rdp_cp_capture_begin(rdp_cp *cp);
int rdp_cp_capture_end(rdp_cp *cp, rdp_graph **out);
/* Replays; when elapsed_ms is non-NULL it receives the GPU time of the replays
 * measured with CUDA events on the processor's stream. */
int rdp_graph_replay(rdp_graph *g, uint32_t count, float *elapsed_ms);
uint32_t rdp_graph_kernel_count(rdp_graph *g);
/* GPU time (ms) of the shading kernel (k_shade, the dominant kernel) in the last replay,
 * from CUDA events recorded on the stream around each of its launches, and their number. */
float rdp_graph_last_shade_ms(rdp_graph *g);
/* The same for the blend kernel (k_blend, whose work queue the learned tile order sorts). */
float rdp_graph_last_blend_ms(rdp_graph *g);
uint32_t rdp_graph_shade_launches(rdp_graph *g);
void rdp_graph_destroy(rdp_graph *g);

/* ---------------------------------------------------------------------------------------------
 * Batched instances.  No single counterpart in the reference, which runs one CommandProcessor
 * per emulator (rdp_device.hpp:111-197); a batch runs many of them on one GPU.  Each instance is
 * an ordinary rdp_cp (every rdp_cp_* call above works on it, with the same results as a
 * stand-alone processor), but its render passes are deferred: rdp_batch_submit launches them for
 * all instances together, one kernel chain per "round" holding the next pass of every instance
 * that has one.  rdp_cp_wait_timeline / rdp_cp_idle / rdp_cp_scanout_sync on an instance submit
 * the batch when they need work that is still deferred.  All instances share the batch's stream
 * and launch buffers; a batch and its instances are used from one thread at a time. */
typedef struct rdp_batch rdp_batch;

enum
{
	RDP_BATCH_TILE_ORDER_LEARNED = 1u << 0, /* start tiles longest-predicted-first (rdp_batch_set_schedule) */
	RDP_BATCH_RECORD_TILE_CYCLES = 1u << 1  /* measure per-tile blend cycles (training data) */
};

typedef struct rdp_batch_create_info
{
	int device;
	uint32_t flags; /* RDP_BATCH_* */
} rdp_batch_create_info;

typedef struct rdp_batch_stats
{
	uint64_t instances;       /* live instances */
	uint64_t rounds;          /* launches of the kernel chain */
	uint64_t passes;          /* passes launched (sum over rounds) */
	uint64_t kernel_launches; /* kernels launched, graph replays included */
	uint64_t staging_bytes;   /* host->device bytes of command/state data */
} rdp_batch_stats;

int rdp_batch_create(const rdp_batch_create_info *info, rdp_batch **out);
/* Destroys the batch; its instances must have been destroyed (rdp_cp_destroy) first. */
int rdp_batch_destroy(rdp_batch *b);
/* Creates an instance of the batch (same arguments and rules as rdp_cp_create). */
int rdp_batch_add_instance(rdp_batch *b, const rdp_create_info *info, rdp_cp **out);
/* Launches every deferred pass of every instance (rounds of at most one pass per instance). */
int rdp_batch_submit(rdp_batch *b);
/* rdp_batch_submit, then waits until the batch's stream is idle. */
int rdp_batch_idle(rdp_batch *b);
int rdp_batch_get_stats(rdp_batch *b, rdp_batch_stats *out);
/* rdp_cp_enqueue for many instances of the batch at once, parsed on `threads` host threads
 * (0: one per core); with timeline_values, each instance is also signalled
 * (rdp_cp_signal_timeline) and its value stored.  Instances must be distinct. */
int rdp_batch_enqueue_many(rdp_batch *b, uint32_t count, rdp_cp *const *instances, const uint32_t *const *words,
                           const uint32_t *num_words, uint64_t *timeline_values, uint32_t threads);
/* Sync-point capture over all instances: between begin and end, deferred passes are recorded
 * (as rdp_cp_capture_begin/end do for one processor) and the graph replays all rounds. */
int rdp_batch_capture_begin(rdp_batch *b);
int rdp_batch_capture_end(rdp_batch *b, rdp_graph **out);

/* Learned tile order.  No counterpart in the reference.  A small MLP (16 -> 64 -> 64 -> 1, ReLU,
 * FP16 weights, FP32 accumulation, RDP_MLP_PARAMS parameters packed as W1[64][16], b1[64],
 * W2[64][64], b2[64], W3[64], b3) predicts each non-empty tile's blend cost from its binning
 * features; the blend kernel then starts tiles longest-predicted-first.  Output never depends
 * on the order.  With `train`, every launch also takes one Adam step (learning_rate) on the
 * launch's tiles (every train_stride-th), target log2(1 + measured blend cycles) / 16.
 * rdp_batch_get_model returns the FP32 parameters and the last step's mean squared error;
 * rdp_batch_set_model loads parameters (and resets the optimiser state). */
#ifndef RDP_MLP_PARAMS
#define RDP_MLP_PARAMS 5313
#endif
int rdp_batch_set_schedule(rdp_batch *b, int learned_order, int train, float learning_rate, uint32_t train_stride);
int rdp_batch_get_model(rdp_batch *b, float *params, float *last_loss);
int rdp_batch_set_model(rdp_batch *b, const float *params);
/* The last launch's non-empty tiles, in tile order: features (16 per tile) and predictions
 * (when the model ran), measured blend cycles (with RDP_BATCH_RECORD_TILE_CYCLES or training).
 * Any output may be NULL; *count receives the number of tiles written (<= max_tiles). */
int rdp_batch_get_tile_samples(rdp_batch *b, float *features, float *predicted, uint32_t *cycles, uint32_t max_tiles,
                               uint32_t *count);
/* The scheduler's GPU kernels on caller data (test and tooling entry points): loss gradients
 * (mean squared error over n samples of RDP_MLP_IN = 16 features) and forward outputs. */
int rdp_mlp_gradients(int device, const float *params, const float *features, const float *targets, uint32_t n,
                      float *grads, float *loss);
int rdp_mlp_forward(int device, const float *params, const float *features, uint32_t n, float *out);

/* Serving loop.  No counterpart in the reference.  Runs a trace of frame requests through a
 * batch with continuous batching: a request arrives at arrival_s (open loop: seconds after the
 * start of the call), waits in arrival order until the frames in flight leave room in the HBM
 * budget (sum of footprint_bytes; 0 = estimated from num_words) and under max_in_flight, is then
 * enqueued to its instance and signalled; every pass of admission is one rdp_batch_submit, so
 * requests admitted while others are on the GPU share the following launches.  A request is
 * complete when its instance's timeline value for it completes (framebuffer copied back to the
 * instance's RDRAM).  All instance state stays resident on the device throughout.  Frames of one
 * instance render in arrival order, so each result equals rendering that instance's requests
 * alone. */
typedef struct rdp_serve_request
{
	uint32_t instance;        /* index into the instances array */
	uint32_t num_words;
	const uint32_t *words;    /* the frame's RDP command words (host memory, alive during the call) */
	double arrival_s;
	uint64_t footprint_bytes; /* transient HBM the frame needs in flight; 0: estimated */
} rdp_serve_request;

typedef struct rdp_serve_config
{
	uint64_t hbm_budget_bytes; /* admission limit on the summed footprint of frames in flight */
	uint32_t max_in_flight;    /* 0: no limit */
	double timeout_s;          /* the call returns RDP_ERR_TIMEOUT after this long */
} rdp_serve_config;

typedef struct rdp_serve_result
{
	double admit_s;   /* admission (enqueue) time */
	double done_s;    /* completion time as seen by the loop */
	double latency_s; /* done_s - arrival_s */
} rdp_serve_result;

typedef struct rdp_serve_stats
{
	uint64_t submits;        /* rdp_batch_submit calls */
	uint64_t max_in_flight;  /* largest number of frames in flight */
	uint64_t max_footprint;  /* largest summed footprint in flight (bytes) */
	double elapsed_s;
} rdp_serve_stats;

int rdp_serve_run(rdp_batch *b, rdp_cp *const *instances, uint32_t num_instances, const rdp_serve_request *requests,
                  uint32_t num_requests, const rdp_serve_config *config, rdp_serve_result *results,
                  rdp_serve_stats *stats);

/* RDPDUMP2 capture files (the reference's format: parallel-rdp/rdp_dump_write.cpp, rdp_dump.cpp).
 * The writer mirrors RDP::RDPDumpWriter (init, flush_dram, flush_hidden_dram, emit_command,
 * set_vi_register, end_frame, signal_complete); rdp_dump_replay plays a file into a processor
 * as the reference's replayer does (replayer_driver_parallel.cpp) and calls on_frame with the
 * RGBA8 scanout of every end-of-frame record. */
typedef struct rdp_dump_writer rdp_dump_writer;
typedef void (*rdp_dump_frame_cb)(void *user, uint32_t frame, const uint32_t *rgba, uint32_t width, uint32_t height);
int rdp_dump_writer_open(const char *path, uint32_t rdram_size, uint32_t hidden_rdram_size, rdp_dump_writer **out);
int rdp_dump_writer_flush_rdram(rdp_dump_writer *w, const void *rdram, uint32_t size);
int rdp_dump_writer_flush_hidden_rdram(rdp_dump_writer *w, const void *hidden, uint32_t size);
int rdp_dump_writer_command(rdp_dump_writer *w, uint32_t op, const uint32_t *words, uint32_t num_words);
int rdp_dump_writer_set_vi_register(rdp_dump_writer *w, uint32_t reg, uint32_t value);
int rdp_dump_writer_end_frame(rdp_dump_writer *w);
int rdp_dump_writer_signal_complete(rdp_dump_writer *w);
int rdp_dump_writer_close(rdp_dump_writer *w);
int rdp_dump_replay(rdp_cp *cp, const char *path, rdp_dump_frame_cb on_frame, void *user, uint32_t *frames);

/* Kernel specialisation.  The reference compiles its shading shaders per normalised static render
 * state with specialisation constants (rdp_renderer.cpp:1294-1331, 1790-1822).  Here the shading
 * kernel is compiled for RDP_SHADE_VARIANTS variants: 0-3 run one general shader for every
 * primitive (2, 3, 4 and 4 (primitive, tile) pairs per warp step, at register budgets for 18, 16, 16
 * and 18 resident CTAs per SM), 4-7 dispatch each primitive to separately compiled code for its
 * render-state class (fill, copy, untextured, one texel, one texel through a TLUT, two texels, LOD;
 * others take the general shader; 2 pairs per step at budgets for 16, 18, 20 and 24 CTAs).  By default
 * an autotuner times them on the first launches of a device and keeps the fastest per shaded
 * (primitive, tile) pair.  All variants give identical results.  rdp_set_shade_variant forces one
 * (0..7) or restarts tuning (-1); rdp_get_shade_variant returns the device's choice, -1 while tuning. */
#define RDP_SHADE_VARIANTS 8
int rdp_set_shade_variant(int device, int variant);
int rdp_get_shade_variant(int device);

/* Order in which k_shade takes the (primitive, tile) pairs of a launch, process-wide per device
 * (default 2, or the RDP_SHADE_ORDER environment variable): 0 = tile order with a fixed stride
 * per CTA, 1 = tile order dealt through one work queue per SM, 2 = primitive-major order dealt
 * through the per-SM queues.  Primitive-major order applies to launches of at least 16,384
 * primitives (RDP_SHADE_PERM_MIN_PRIMS), the queues to launches of at least 64 pairs per CTA
 * (RDP_SHADE_QUEUE_MIN); smaller launches take the next simpler order.  The variables are read
 * when a processor or batch is created.  All orders give identical results. */
int rdp_set_shade_order(int device, int order);
int rdp_get_shade_order(int device);

/* ---------------------------------------------------------------------------------------------
 * Allocation-free TMEM update.  No counterpart in the reference: it exists for callers that must
 * not allocate device memory -- for example an emulator frame loop that runs inside a CUDA stream
 * capture (cudaMalloc is not allowed while a stream is being captured) or that must never stall on
 * cudaMalloc/cudaFree, or a host application that owns all device memory through its own
 * allocator and hands this library finished buffers only.
 *
 * It applies `num_uploads` TMEM upload descriptors to `tmem` (2048 16-bit words, updated in place),
 * reading texels from `rdram`, and writes the TMEM image after each upload to `snapshots`
 * ((num_uploads + 1) x 2048 words; snapshot 0 is the TMEM on entry).  All pointers are device
 * pointers owned by the caller; the work is queued on `stream` (a cudaStream_t, NULL for the
 * legacy stream) and the call returns without waiting.
 *
 * The stage's scratch bitmask lives in a fixed device array inside this library (256 KiB, held by
 * every GPU that loads the library until the process exits), so num_uploads is limited to
 * RDP_NOALLOC_MAX_UPLOADS; larger requests return RDP_ERR_TOO_LARGE without doing anything.
 * The first call on each device looks up that array's device address (with the device current);
 * make that first call before starting any stream capture.  All calls on a device share that
 * device's one array and it keeps the last call's contents, so calls whose GPU work overlaps in
 * time on the same device (for example on two streams) race: order them on one stream.  No call
 * allocates memory. */
#define RDP_NOALLOC_MAX_UPLOADS 1024

/* One TMEM upload plan, 64 bytes: the region of RDRAM a texture load reads and where in TMEM it
 * lands, as this library's command processor derives it from a LoadTile / LoadTLUT / LoadBlock
 * command and the tile descriptor it names. */
typedef struct rdp_tmem_upload
{
	int32_t width, height;                 /* texels per line written to TMEM (rounded to whole words), lines */
	float min_t_mod, max_t_mod;            /* LoadBlock: reciprocals of the longest and shortest line lengths */
	int32_t vram_addr;                     /* RDRAM byte address of the first texel */
	int32_t vram_width;                    /* texels per RDRAM line */
	int32_t vram_size;                     /* RDRAM texel size: 1 = 8, 2 = 16, 3 = 32 bits */
	int32_t vram_effective_width;          /* texels per line actually read (rounded to 64-bit words) */
	int32_t tmem_offset;                   /* TMEM byte offset of the first line */
	int32_t tmem_stride_words;             /* TMEM line stride in 16-bit words (LoadBlock: in 64-bit words) */
	int32_t tmem_size, tmem_fmt;           /* the tile descriptor's texel size and format */
	int32_t mode;                          /* 0 LoadTile, 1 LoadTLUT, 2 LoadBlock */
	float inv_tmem_stride_words;           /* 1 / tmem_stride_words, rounded to fp32 on the host */
	int32_t dxt;                           /* LoadBlock: line step in 1/65536 lines per 64-bit word */
	int32_t padding;
} rdp_tmem_upload;

int rdp_tmem_update_noalloc(const rdp_tmem_upload *uploads, uint32_t num_uploads, const uint8_t *rdram,
                            uint32_t rdram_size, uint16_t *tmem, uint16_t *snapshots, void *stream);

#ifdef __cplusplus
}
#endif
#endif
