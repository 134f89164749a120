/*
 * Host side of the GB300 RDP path: the command processor behind the C ABI
 * (include/rdp_cuda.h), replacing RDP::CommandProcessor + RDP::Renderer
 * (parallel-rdp/rdp_device.cpp, parallel-rdp/rdp_renderer.cpp).
 *
 * The host performs only the sequential part of command processing:
 *   - splits the word stream into commands (RDP command lengths),
 *   - keeps the state registers as raw words (state blocks) -- decoding them is
 *     done per primitive on the GPU,
 *   - decodes tile descriptors and plans TMEM uploads (load_tile,
 *     rdp_renderer.cpp:3099-3486), which depend on the order of loads,
 *   - segments the stream into passes on framebuffer changes, TMEM loads that
 *     read pending framebuffer writes (rdp_renderer.cpp:3051-3097), SyncFull and
 *     capacity limits, and
 *   - owns RDRAM coherency and the timeline.
 * One pass is one H2D copy of a packed staging buffer plus four kernel
 * launches on the processor's stream.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <deque>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/rdp_cuda.h"
#include "rdp_types.h"
#include "rdp_kernels.h"
#include "rdp_exec.h"
#include "sched.h"
#include <cuda_fp16.h>
#include "vi.h"
#include "rdp_coherency.h"
#include "rdp_upscale.h"
#include "blender_divider_runs.inc"

namespace {

constexpr uint32_t kMaxWordsPerPass = RDP_MAX_PRIMS_PER_PASS * 44;
constexpr uint32_t kMaxStateBlocks = RDP_MAX_PRIMS_PER_PASS;
constexpr uint32_t kMaxTilesets = 32768;
// Primitives after which (and every as many after) a stand-alone processor's pass goes to an idle GPU.
constexpr size_t kEagerFlushPrims = 4096;
constexpr uint32_t kMaxTiles = RDP_MAX_TILES_X * RDP_MAX_TILES_Y;


// Words of a command (rdp_device.cpp command lengths); the in-band meta ops share the stream
// (rdp_common.hpp:37-43): MetaSignalTimeline carries a 64-bit value, MetaFlush and MetaIdle are
// one word, MetaSetQuirks two.
static uint32_t command_length(uint32_t op)
{
	switch (op)
	{
	case 0x01: return 3;
	case 0x02:
	case 0x03: return 1;
	case 0x08: return 8;
	case 0x09: return 12;
	case 0x0a: return 24;
	case 0x0b: return 28;
	case 0x0c: return 24;
	case 0x0d: return 28;
	case 0x0e: return 40;
	case 0x0f: return 44;
	case 0x24:
	case 0x25: return 4;
	default: return 2;
	}
}

static int sext(uint32_t v, int bits) { return int(v << (32 - bits)) >> (32 - bits); }

// Blender divider table: floor(n / d) & 0xff except for the irregular entries stored as runs.
static void build_blender_lut(uint8_t *lut)
{
	for (int d = 0; d < 16; d++)
		for (int n = 0; n < 2048; n++)
			lut[(d << 11) | n] = d ? uint8_t((n / d) & 0xff) : 0;
	for (int i = 0; i < RDP_BLENDER_DIVIDER_NUM_RUNS; i++)
	{
		const unsigned short *r = rdp_blender_divider_runs[i];
		for (int k = 0; k < r[2]; k++) lut[(r[0] << 11) | (r[1] + k)] = uint8_t(r[3]);
	}
}

std::mutex g_lut_mutex;
std::vector<int> g_lut_devices;

static cudaError_t ensure_luts(int device)
{
	std::lock_guard<std::mutex> hold(g_lut_mutex);
	for (int d : g_lut_devices)
		if (d == device) return cudaSuccess;
	static uint8_t lut[0x8000];
	build_blender_lut(lut);
	cudaError_t e = rdp_kernels_init_luts(lut);
	if (e == cudaSuccess) g_lut_devices.push_back(device);
	return e;
}

// The command thread's ring (command_ring.cpp:71-134): the emulator thread pushes command words,
// blocking while the ring is full; one worker thread decodes them in order.  drain() returns once
// every pushed word has been decoded.  A chunk longer than the ring is pushed in pieces (the
// decoder carries a partial command over to the next piece).
class CommandRing
{
public:
	static constexpr uint32_t kWords = 4096;

	void start(std::function<void(uint32_t, const uint32_t *)> consume)
	{
		consume_ = std::move(consume);
		ring_.assign(kWords, 0u);
		worker_ = std::thread([this] { loop(); });
	}

	void push(uint32_t n, const uint32_t *w)
	{
		while (n)
		{
			const uint32_t k = std::min<uint32_t>(n, kWords - 1);
			std::unique_lock<std::mutex> lk(mu_);
			cv_.wait(lk, [&] { return write_ + k + 1 <= read_ + kWords; });
			ring_[write_++ % kWords] = k;
			for (uint32_t i = 0; i < k; i++) ring_[write_++ % kWords] = w[i];
			cv_.notify_all();
			n -= k;
			w += k;
		}
	}

	void drain()
	{
		std::unique_lock<std::mutex> lk(mu_);
		cv_.wait(lk, [&] { return completed_ == write_; });
	}

	// Waits until pred() holds (checked after each decoded chunk) or the deadline passes.
	template <class Pred>
	bool wait_until(Pred pred, std::chrono::steady_clock::time_point deadline, bool bounded)
	{
		std::unique_lock<std::mutex> lk(mu_);
		if (!bounded)
		{
			cv_.wait(lk, pred);
			return true;
		}
		return cv_.wait_until(lk, deadline, pred);
	}

	void stop()
	{
		if (!worker_.joinable()) return;
		{
			std::lock_guard<std::mutex> lk(mu_);
			stop_ = true;
		}
		cv_.notify_all();
		worker_.join();
	}

	std::mutex &mutex() { return mu_; }

private:
	void loop()
	{
		std::vector<uint32_t> chunk;
		for (;;)
		{
			{
				std::unique_lock<std::mutex> lk(mu_);
				cv_.wait(lk, [&] { return stop_ || write_ > read_; });
				if (write_ == read_ && stop_) return;
				const uint32_t k = ring_[read_++ % kWords];
				chunk.resize(k);
				for (uint32_t i = 0; i < k; i++) chunk[i] = ring_[read_++ % kWords];
				cv_.notify_all(); // room for the producer
			}
			consume_(uint32_t(chunk.size()), chunk.data());
			std::lock_guard<std::mutex> lk(mu_);
			completed_ = read_;
			cv_.notify_all();
		}
	}

	std::function<void(uint32_t, const uint32_t *)> consume_;
	std::vector<uint32_t> ring_;
	uint64_t write_ = 0, read_ = 0, completed_ = 0;
	bool stop_ = false;
	std::mutex mu_;
	std::condition_variable cv_;
	std::thread worker_;
};

// Builds the page lists of the coherency kernels (coherency.cu) for any number of instances and
// pages, launching a list whenever its instance slots or pages are full.
class CohLauncher
{
public:
	void add(uint8_t *host, uint8_t *dev, uint32_t *wmask, uint32_t page)
	{
		if (slot_ < 0 || L_.host[slot_] != host)
		{
			if (slots_used_ == RDP_COH_MAX_INSTANCES) flush_list();
			slot_ = slots_used_++;
			L_.host[slot_] = host;
			L_.dev[slot_] = dev;
			L_.wmask[slot_] = wmask;
			if ((reinterpret_cast<uintptr_t>(host) & 15u) == 0) L_.host_aligned |= 1u << slot_;
		}
		L_.entry[L_.count++] = (uint32_t(slot_) << 24) | page;
		if (L_.count == RDP_COH_MAX_PAGES)
		{
			const int keep = slot_;
			uint8_t *h = L_.host[keep], *d = L_.dev[keep];
			uint32_t *m = L_.wmask[keep];
			flush_list();
			slot_ = slots_used_++;
			L_.host[slot_] = h;
			L_.dev[slot_] = d;
			L_.wmask[slot_] = m;
			if ((reinterpret_cast<uintptr_t>(h) & 15u) == 0) L_.host_aligned |= 1u << slot_;
		}
	}
	// Launches what is left; returns the first launch error.
	cudaError_t finish(cudaStream_t stream, int to_host)
	{
		stream_ = stream;
		to_host_ = to_host;
		flush_list();
		return err_;
	}
	void begin(cudaStream_t stream, int to_host)
	{
		stream_ = stream;
		to_host_ = to_host;
	}

private:
	void flush_list()
	{
		if (L_.count && err_ == cudaSuccess) err_ = rdp_coherency_launch(&L_, to_host_, stream_);
		L_.count = 0;
		L_.host_aligned = 0;
		slots_used_ = 0;
		slot_ = -1;
	}
	RdpCohList L_ = {};
	int slots_used_ = 0, slot_ = -1, to_host_ = 0;
	cudaStream_t stream_ = nullptr;
	cudaError_t err_ = cudaSuccess;
};

} // namespace

namespace rdpx {
// RDP_SHADE_VARIANT=<0..3> in the environment fixes the variant (profiling, experiments).
int &shade_order_choice(int device)
{
	static std::vector<int> choice = [] {
		int v = 2;
		if (const char *e = getenv("RDP_SHADE_ORDER"))
		{
			int x = atoi(e);
			if (x >= 0 && x <= 2) v = x;
		}
		return std::vector<int>(64, v);
	}();
	return choice[device >= 0 && device < 64 ? device : 0];
}

int &shade_variant_choice(int device)
{
	static std::vector<int> choice = [] {
		int v = -1;
		if (const char *e = getenv("RDP_SHADE_VARIANT"))
		{
			int x = atoi(e);
			if (x >= 0 && x < RDP_SHADE_VARIANTS) v = x;
		}
		return std::vector<int>(64, v);
	}();
	return choice[device >= 0 && device < 64 ? device : 0];
}
} // namespace rdpx

struct rdp_batch;

struct rdp_cp
{
	// ---------------------------------------------------------------- configuration
	int device = 0;
	cudaStream_t stream = nullptr;
	uint8_t *host_rdram = nullptr;
	bool own_host_rdram = false;
	bool host_registered = false;
	uint32_t rdram_size = 0, hidden_size = 0;
	std::vector<uint8_t> hidden_mirror;

	// ---------------------------------------------------------------- device memory
	// The instance's own state; launch buffers belong to the executor.
	uint8_t *d_rdram = nullptr, *d_hidden = nullptr;
	uint16_t *d_tmem = nullptr, *d_snapshots = nullptr;
	unsigned long long *d_fragments = nullptr; // [0] fragments, [1] touched tiles, [2] tile instances
	rdpx::Executor own_exec;
	rdpx::Executor *exec = &own_exec;
	rdp_batch *batch = nullptr;
	std::deque<rdpx::PassPacket> deferred;   // batched: passes waiting for the batch's next launch
	std::vector<uint64_t> unsubmitted;       // batched: timeline values signalled before that launch

	// ---------------------------------------------------------------- internal upscaling
	// RDP_CREATE_UPSCALING_* (Renderer::init_internal_upscaling_factor, rdp_renderer.cpp:545-601):
	// the multisampled copy of RDRAM and hidden RDRAM (factor^2 slices each, then the super-sampled
	// write mask) and the reference copy of what it reflects of RDRAM.
	uint32_t up_log2 = 0;
	bool ssaa = false, ssaa_dither = false;
	uint8_t *d_ms_rdram = nullptr, *d_ms_hidden = nullptr, *d_up_reference = nullptr;
	static constexpr size_t kSsaaMaskBytes = 2 * 1024 * 1024 / 8; // 2 bits per pixel of a 1024 x 1024 image
	RdpUpscaleDomain up_domain() const
	{
		RdpUpscaleDomain d = {};
		d.rdram = d_rdram;
		d.hidden = d_hidden;
		d.reference = d_up_reference;
		d.ms_rdram = d_ms_rdram;
		d.ms_hidden = d_ms_hidden;
		d.ssaa_mask = ssaa ? reinterpret_cast<uint32_t *>(d_ms_rdram + (size_t(rdram_size) << (2 * up_log2))) : nullptr;
		d.wmask = coherent ? d_wmask : nullptr;
		d.rdram_size = rdram_size;
		d.hidden_size = hidden_size;
		d.samples = 1u << (2 * up_log2);
		return d;
	}

	// ---------------------------------------------------------------- pass being recorded
	std::vector<RdpPrimIn> prims;
	std::vector<RdpPrimIn> grouped; // prims regrouped by target at flush
	std::vector<uint32_t> words;
	std::vector<uint32_t> state_blocks;
	std::vector<RdpTile> tilesets;
	std::vector<RdpUpload> uploads;

	// ---------------------------------------------------------------- register state
	uint32_t sb[RDP_STATE_BLOCK_WORDS] = {};
	bool sb_dirty = true;
	RdpTile tiles[8] = {};
	bool tiles_dirty = true;
	struct { uint32_t addr = 0, width = 0, size = 0, fmt = 0; } tex_image;
	struct
	{
		uint32_t addr = 0, width = 0, fmt = FBF_RGBA5551, depth_addr = 0;
	} fb; // image registers (SetColorImage / SetMaskImage)
	uint64_t base_prim_index = 0;
	std::vector<uint32_t> carry;

	// A pass may draw into several colour images ("targets") as long as their memory --
	// colour, and depth where a target uses it -- does not overlap: their pixels are then
	// independent and the order between them does not matter.  The reference ends its pass
	// at every image change; it keeps pixel state for the pass (init_tile/finish_tile,
	// memory_interfacing.h:286-362), and for RGBA5551, RGBA8888, IA88 and I4 images that
	// store/reload round trip is transparent, so longer passes give identical results.
	struct Target
	{
		uint32_t addr = 0, width = 0, fmt = 0, depth_addr = 0, deduced_height = 0;
		uint32_t span_prims = 0;        // primitives with span rows (the reference's span jobs)
		bool color_pending = false, depth_pending = false, depth_used = false;
		std::vector<uint32_t> prim_ids; // indices into `prims`
	};
	std::vector<Target> targets;
	bool pass_fill_only = true; // every primitive of the pass is drawn by the fill pipe (cycle type 3)

	// The reference's own pass (it ends after 256 primitives, before the 256th TMEM upload,
	// at image changes, load hazards and SyncFull; rdp_renderer.cpp:1564-1590, 3051-3097,
	// 3484-3485): the state its load-hazard check sees.  For I8 images and colour/depth
	// aliasing the round trip is NOT transparent (odd I8 pixels store green but blending
	// reads red; aliased colour and depth share memory), so there the passes of this
	// processor end exactly where the reference's do.
	struct RefView
	{
		uint32_t prims = 0, uploads = 0, deduced_height = 0;
		bool color_pending = false, depth_pending = false;
	} rv;
	static bool boundaries_visible(uint32_t fmt, uint32_t addr, uint32_t depth_addr)
	{
		return fmt == FBF_I8 || addr == depth_addr;
	}
	// With upscaling every pass is the reference's pass: its pre / post updates of the upscaled
	// domain follow the reference's pass boundaries.
	bool pass_boundaries_visible() const { return up_log2 || boundaries_visible(fb.fmt, fb.addr, fb.depth_addr); }
	// The reference's pass ends: with visible boundaries this processor's pass ends too.
	void rv_end()
	{
		rv = RefView{};
		if (pass_boundaries_visible()) flush();
	}

	// ---------------------------------------------------------------- coherency + timeline
	std::vector<std::pair<uint32_t, uint32_t>> dirty_ranges;
	bool host_rdram_dirty = false;
	// Page-granular coherency with the caller's RDRAM when it is mapped into the device's address
	// space (rdp_renderer.cpp:2523-2907): every pass first refreshes the pages it reads from the
	// host (masked: bytes the GPU wrote and has not yet returned stay), and a timeline value writes
	// the bytes the GPU wrote back into the host pages (masked: other bytes stay the caller's).
	bool coherent = false;
	uint8_t *host_mapped = nullptr;    // host_rdram's address in the device's address space
	uint32_t *d_wmask = nullptr;       // 1 bit per RDRAM byte written by the GPU, not yet returned
	std::vector<uint8_t> page_written; // pages holding such bytes
	std::vector<uint32_t> page_stamp;  // last pass that listed a page for refresh
	uint32_t stamp = 0;
	std::vector<uint32_t> read_pages;  // pages the pass being recorded reads
	bool refresh_all = false;          // end_write_rdram: every page is refreshed before the next pass
	uint64_t timeline_counter = 0;
	std::deque<std::pair<uint64_t, cudaEvent_t>> pending;
	std::vector<cudaEvent_t> free_events;
	uint64_t completed_value = 0;

	// ---------------------------------------------------------------- statistics
	rdp_stats stats = {};
	struct
	{
		uint32_t prims = 0, uploads = 0, span_jobs = 0;
		std::vector<uint64_t> static_keys, depth_keys;
	} ref;

	// Sync-point capture: recorded launches with device-resident inputs.  capture_written keeps
	// the RDRAM ranges the recorded passes write: every replay of the graph writes them again, so
	// the replay marks them for copy-back like a pass does.
	bool capturing = false;
	rdpx::CaptureSink capture_sink;
	std::vector<std::pair<uint32_t, uint32_t>> capture_written;
	bool in_capture() const; // this processor's passes are being recorded (its own or its batch's capture)

	uint32_t vi_regs[16] = {};
	struct ViHost
	{
		// Per-scanline registers (video_interface.cpp:1102-1213).
		uint32_t flags = 0;
		bool ended = false;
		unsigned line = 0;
		uint32_t hs_latched = 0, xs_latched = 0;
		uint32_t hs_line[640] = {}, xs_line[640] = {};
		// Frame state (video_interface.hpp:149-161).
		bool previous_frame_blank = false;
		uint32_t frame_count = 0, last_valid_frame_count = 0;
		bool have_prev = false;
		int prev_w = 0, prev_h = 0;
		// Device images.
		uint32_t *d_aa = nullptr, *d_dv = nullptr, *d_out[2] = { nullptr, nullptr };
		uint32_t *d_half = nullptr; // downscale step output
		size_t half_cap = 0;
		size_t aa_cap = 0, dv_cap = 0;
		int cur = 0;
		RdpViLine *d_lines = nullptr, *h_lines = nullptr;
		cudaEvent_t lines_copied = nullptr;
		bool tables = false;
	} vi;
	rdp_validation_cb validation_cb = nullptr;
	void *validation_user = nullptr;
	int sticky_error = RDP_OK;

	// Command thread (RDP_CREATE_COMMAND_THREAD): the C ABI pushes words into the ring and the
	// worker decodes them; timeline values are handed out by the caller (api_value) and travel
	// in band (MetaSignalTimeline), decoded_value is the last one the worker has reached.  The
	// pending-event list is shared between the worker (signal) and the waiting caller.
	CommandRing *ring = nullptr;
	uint64_t api_value = 0;
	std::atomic<uint64_t> decoded_value{ 0 };
	std::mutex timeline_mu;

	// ================================================================= helpers
	void report(int err, const char *msg)
	{
		if (validation_cb) validation_cb(validation_user, err, msg);
	}

	int check(cudaError_t e)
	{
		if (e != cudaSuccess)
		{
			sticky_error = RDP_ERR_DEVICE;
			return RDP_ERR_DEVICE;
		}
		return RDP_OK;
	}

	uint32_t cycle_type() const { return (sb[SB_OTHER_MODES] >> 20) & 3; }

	// Emulation of the reference's pass segmentation for the reference_passes counter
	// (need_flush rdp_renderer.cpp:1564-1590 and the upload limit at 3484-3485).
	void ref_pass_break()
	{
		stats.reference_passes++;
		ref.prims = ref.uploads = ref.span_jobs = 0;
		ref.static_keys.clear();
		ref.depth_keys.clear();
	}
	void ref_note_prim(int lines)
	{
		uint64_t skey = (uint64_t(sb[SB_OTHER_MODES]) << 32) ^ (uint64_t(sb[SB_OTHER_MODES + 1] & 0x3f0fu) << 20) ^
		                uint64_t(sb[SB_COMBINE]) ^ (uint64_t(sb[SB_COMBINE + 1]) << 7);
		uint64_t dkey = (uint64_t(sb[SB_OTHER_MODES + 1]) << 8) | ((sb[SB_OTHER_MODES] >> 20) & 3);
		if (std::find(ref.static_keys.begin(), ref.static_keys.end(), skey) == ref.static_keys.end())
			ref.static_keys.push_back(skey);
		if (std::find(ref.depth_keys.begin(), ref.depth_keys.end(), dkey) == ref.depth_keys.end())
			ref.depth_keys.push_back(dkey);
		ref.prims++;
		if (lines > 0) ref.span_jobs += uint32_t((lines + 2 + 63) / 64);
		if (ref.prims >= 256 || ref.static_keys.size() >= 64 || ref.depth_keys.size() >= 64 ||
		    ref.span_jobs * 64 + 1024 > 32 * 1024)
			ref_pass_break();
	}

	// ================================================================= creation
	// `shared` is the batch's executor (whose stream the instance then uses), or null.
	int init(const rdp_create_info *info, rdp_batch *owner = nullptr, rdpx::Executor *shared = nullptr)
	{
		device = info->device;
		rdram_size = uint32_t(info->rdram_size);
		hidden_size = uint32_t(info->hidden_rdram_size);
		if (cudaSetDevice(device) != cudaSuccess) return RDP_ERR_UNSUPPORTED;
		if (ensure_luts(device) != cudaSuccess) return RDP_ERR_DEVICE;
		if (owner)
		{
			batch = owner;
			exec = shared;
			stream = shared->stream;
		}
		else if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess)
			return RDP_ERR_DEVICE;

		if (info->rdram)
			host_rdram = static_cast<uint8_t *>(info->rdram) + info->rdram_offset;
		else
		{
			host_rdram = static_cast<uint8_t *>(calloc(1, rdram_size));
			if (!host_rdram) return RDP_ERR_OOM;
			own_host_rdram = true;
		}
		host_registered = cudaHostRegister(host_rdram, rdram_size, cudaHostRegisterMapped) == cudaSuccess;
		if (!host_registered) cudaGetLastError();
		if (host_registered && rdram_size >= RDP_RDRAM_PAGE_BYTES &&
		    cudaHostGetDevicePointer(reinterpret_cast<void **>(&host_mapped), host_rdram, 0) == cudaSuccess)
			coherent = true;
		cudaGetLastError();
		hidden_mirror.assign(hidden_size, 0x03);

		if (cudaMalloc(&d_rdram, rdram_size) != cudaSuccess) return RDP_ERR_OOM;
		if (cudaMalloc(&d_hidden, hidden_size) != cudaSuccess) return RDP_ERR_OOM;
		if (cudaMalloc(&d_tmem, 4096) != cudaSuccess) return RDP_ERR_OOM;
		if (cudaMalloc(&d_snapshots, size_t(RDP_MAX_UPLOADS_PER_PASS + 1) * 4096) != cudaSuccess) return RDP_ERR_OOM;
		if (cudaMalloc(&d_fragments, 4 * sizeof(unsigned long long)) != cudaSuccess) return RDP_ERR_OOM;
		if (coherent)
		{
			if (cudaMalloc(&d_wmask, rdram_size / 8) != cudaSuccess) return RDP_ERR_OOM;
			if (check(cudaMemsetAsync(d_wmask, 0, rdram_size / 8, stream))) return RDP_ERR_DEVICE;
			page_written.assign(rdram_size / RDP_RDRAM_PAGE_BYTES, 0);
			page_stamp.assign(rdram_size / RDP_RDRAM_PAGE_BYTES, 0);
		}
		if (!batch)
		{
			// A stand-alone processor sizes its executor for one full pass up front.
			rdpx::ExecCaps c;
			c.passes = 1;
			c.prims = RDP_MAX_PRIMS_PER_PASS;
			c.uploads = RDP_MAX_UPLOADS_PER_PASS;
			c.tile_items = kMaxTiles;
			c.staging = rdpx::align16(sizeof(RdpPass)) + rdpx::align16(sizeof(RdpPrimIn) * RDP_MAX_PRIMS_PER_PASS) +
			            rdpx::align16(sizeof(uint32_t) * kMaxWordsPerPass) +
			            rdpx::align16(sizeof(uint32_t) * RDP_STATE_BLOCK_WORDS * kMaxStateBlocks) +
			            rdpx::align16(sizeof(RdpTile) * 8 * kMaxTilesets) +
			            rdpx::align16(sizeof(RdpUpload) * RDP_MAX_UPLOADS_PER_PASS) + 512;
			if (!own_exec.init(device, stream)) return RDP_ERR_OOM;
			c.pairs = own_exec.initial_pairs;
			c.span_rows = own_exec.initial_span_rows;
			if (!own_exec.ensure(c)) return RDP_ERR_OOM;
		}
		if (check(cudaMemsetAsync(d_hidden, 0x03, hidden_size, stream))) return RDP_ERR_DEVICE;
		if (check(cudaMemsetAsync(d_tmem, 0, 4096, stream))) return RDP_ERR_DEVICE;
		const uint32_t up = info->flags & (RDP_CREATE_UPSCALING_2X | RDP_CREATE_UPSCALING_4X | RDP_CREATE_UPSCALING_8X);
		if (up)
		{
			// The largest factor asked for wins (rdp_device.cpp:189-196).
			up_log2 = (up & RDP_CREATE_UPSCALING_8X) ? 3 : (up & RDP_CREATE_UPSCALING_4X) ? 2 : 1;
			ssaa = (info->flags & RDP_CREATE_SUPER_SAMPLED_READ_BACK) != 0;
			ssaa_dither = ssaa && (info->flags & RDP_CREATE_SUPER_SAMPLED_DITHER) != 0;
			const size_t n = size_t(1) << (2 * up_log2);
			const size_t ms_bytes = n * rdram_size + (ssaa ? kSsaaMaskBytes : 0);
			if (cudaMalloc(&d_ms_rdram, ms_bytes) != cudaSuccess) return RDP_ERR_OOM;
			if (cudaMalloc(&d_ms_hidden, n * hidden_size) != cudaSuccess) return RDP_ERR_OOM;
			if (cudaMalloc(&d_up_reference, rdram_size) != cudaSuccess) return RDP_ERR_OOM;
			if (check(cudaMemsetAsync(d_ms_rdram, 0, ms_bytes, stream)) ||
			    check(cudaMemsetAsync(d_ms_hidden, 0x03, n * hidden_size, stream)) ||
			    check(cudaMemsetAsync(d_up_reference, 0, rdram_size, stream)))
				return RDP_ERR_DEVICE;
		}
		if (check(cudaMemsetAsync(d_fragments, 0, 4 * sizeof(unsigned long long), stream))) return RDP_ERR_DEVICE;
		if (check(cudaMemcpyAsync(d_rdram, host_rdram, rdram_size, cudaMemcpyHostToDevice, stream))) return RDP_ERR_DEVICE;
		if (check(cudaStreamSynchronize(stream))) return RDP_ERR_DEVICE;

		// Default register state matches a freshly constructed CommandProcessor.
		sb[SB_QUIRKS] = 1; // native_resolution_tex_rect (rdp_device.hpp:79-83)
		for (auto &t : tiles) t = RdpTile{};
		prims.reserve(RDP_MAX_PRIMS_PER_PASS);
		words.reserve(1 << 16);
		return RDP_OK;
	}

	void destroy()
	{
		if (stream)
		{
			cudaSetDevice(device);
			cudaStreamSynchronize(stream);
		}
		for (auto &p : pending) cudaEventDestroy(p.second);
		for (auto e : free_events) cudaEventDestroy(e);
		if (!batch) own_exec.destroy();
		deferred.clear();
		cudaFree(d_rdram);
		cudaFree(d_hidden);
		cudaFree(d_tmem);
		cudaFree(d_snapshots);
		cudaFree(d_fragments);
		cudaFree(d_wmask);
		cudaFree(d_ms_rdram);
		cudaFree(d_ms_hidden);
		cudaFree(d_up_reference);
		cudaFree(vi.d_aa);
		cudaFree(vi.d_dv);
		cudaFree(vi.d_out[0]);
		cudaFree(vi.d_out[1]);
		cudaFree(vi.d_half);
		cudaFree(vi.d_lines);
		if (vi.h_lines) cudaFreeHost(vi.h_lines);
		if (vi.lines_copied) cudaEventDestroy(vi.lines_copied);
		if (host_registered) cudaHostUnregister(host_rdram);
		if (own_host_rdram) free(host_rdram);
		if (stream && !batch) cudaStreamDestroy(stream);
	}

	// ================================================================= pass submission
	static uint32_t bytes_per_pixel(uint32_t fmt)
	{
		switch (fmt)
		{
		case FBF_I4:
		case FBF_I8: return 1;
		case FBF_RGBA8888: return 4;
		default: return 2;
		}
	}

	// RDRAM byte range [lo, hi) of `rows` rows of a target's colour (or depth) image;
	// ranges that wrap around RDRAM cover all of it.
	std::pair<uint64_t, uint64_t> image_range(uint32_t addr, uint32_t width, uint32_t bpp, uint32_t rows) const
	{
		uint64_t lo = addr & (rdram_size - 1), hi = lo + uint64_t(width) * rows * bpp;
		if (hi > rdram_size) return { 0, rdram_size };
		return { lo, hi };
	}
	static bool overlap(std::pair<uint64_t, uint64_t> a, std::pair<uint64_t, uint64_t> b)
	{
		return a.first < a.second && b.first < b.second && a.first < b.second && b.first < a.second;
	}
	// Would target `ti`, grown to `rows` rows (using depth if `depth`), touch memory that
	// another target of the pass touches?
	bool target_conflicts(size_t ti, uint32_t rows, bool depth) const
	{
		const Target &n = targets[ti];
		auto nc = image_range(n.addr, n.width, bytes_per_pixel(n.fmt), rows);
		std::pair<uint64_t, uint64_t> nd = { 0, 0 };
		if (depth || n.depth_used) nd = image_range(n.depth_addr, n.width, 2, rows);
		for (size_t k = 0; k < targets.size(); k++)
		{
			if (k == ti) continue;
			const Target &o = targets[k];
			auto oc = image_range(o.addr, o.width, bytes_per_pixel(o.fmt), o.deduced_height);
			std::pair<uint64_t, uint64_t> od = { 0, 0 };
			if (o.depth_used) od = image_range(o.depth_addr, o.width, 2, o.deduced_height);
			if (overlap(nc, oc) || overlap(nc, od) || overlap(nd, oc) || overlap(nd, od)) return true;
		}
		return false;
	}

	void add_dirty(uint32_t addr, uint32_t bytes)
	{
		if (!bytes) return;
		addr &= rdram_size - 1;
		uint32_t end = std::min<uint64_t>(uint64_t(addr) + bytes, rdram_size);
		if (in_capture()) capture_written.emplace_back(addr, end);
		if (coherent) mark_written_range(addr, end);
		else merge_dirty(addr, end);
	}
	// Pages of RDRAM bytes [addr, addr + bytes), wrapping around RDRAM.
	template <class F> void for_pages(uint64_t addr, uint64_t bytes, F f) const
	{
		if (!bytes) return;
		const uint32_t np = rdram_size / RDP_RDRAM_PAGE_BYTES;
		uint64_t first = (addr & (rdram_size - 1)) / RDP_RDRAM_PAGE_BYTES;
		uint64_t count = ((addr & (RDP_RDRAM_PAGE_BYTES - 1)) + bytes + RDP_RDRAM_PAGE_BYTES - 1) / RDP_RDRAM_PAGE_BYTES;
		if (count > np) count = np;
		for (uint64_t k = 0; k < count; k++) f(uint32_t((first + k) % np));
	}
	void mark_written_range(uint32_t addr, uint32_t end)
	{
		for_pages(addr, uint64_t(end) - addr, [&](uint32_t pg) { page_written[pg] = 1; });
	}
	void mark_read_range(uint64_t addr, uint64_t bytes)
	{
		for_pages(addr, bytes, [&](uint32_t pg) {
			if (page_stamp[pg] != stamp)
			{
				page_stamp[pg] = stamp;
				read_pages.push_back(pg);
			}
		});
	}
	// The pages the recorded pass reads: its texture sources and its images.
	void begin_page_list()
	{
		read_pages.clear();
		if (++stamp == 0)
		{
			std::fill(page_stamp.begin(), page_stamp.end(), 0u);
			stamp = 1;
		}
	}
	void collect_read_pages()
	{
		begin_page_list();
		if (refresh_all)
		{
			mark_read_range(0, rdram_size);
			refresh_all = false;
			return;
		}
		for (const RdpUpload &u : uploads)
		{
			const uint64_t bpt = u.vram_size >= 1 ? (uint64_t(1) << (u.vram_size - 1)) : 1;
			const uint64_t lines = u.mode == 2 ? 1 : uint64_t(std::max(u.height, 1));
			const uint64_t span = ((lines - 1) * uint64_t(std::max(u.vram_width, 0)) +
			                       uint64_t(std::max(u.vram_effective_width, u.width))) * bpt + 8;
			mark_read_range(uint32_t(u.vram_addr), span);
		}
		for (const Target &tg : targets)
		{
			if (!tg.width || !tg.deduced_height || tg.prim_ids.empty()) continue;
			mark_read_range(tg.addr, uint64_t(tg.width) * tg.deduced_height * bytes_per_pixel(tg.fmt));
			if (tg.depth_used || tg.depth_pending) mark_read_range(tg.depth_addr, uint64_t(tg.width) * tg.deduced_height * 2);
		}
	}
	// Queues the masked host -> device refresh of the listed pages on the stream.
	int refresh_pages(const std::vector<uint32_t> &pages)
	{
		if (pages.empty()) return RDP_OK;
		CohLauncher cl;
		cl.begin(stream, 0);
		for (uint32_t pg : pages) cl.add(host_mapped, d_rdram, d_wmask, pg);
		return check(cl.finish(stream, 0));
	}
	// Queues the masked write-back of every page with GPU writes; `cl` collects pages of several
	// instances when given.
	void write_back_pages(CohLauncher &cl)
	{
		for (size_t pg = 0; pg < page_written.size(); pg++)
			if (page_written[pg])
			{
				cl.add(host_mapped, d_rdram, d_wmask, uint32_t(pg));
				page_written[pg] = 0;
			}
	}
	void merge_dirty(uint32_t addr, uint32_t end)
	{
		for (auto &r : dirty_ranges)
		{
			if (addr <= r.second && end >= r.first)
			{
				r.first = std::min(r.first, addr);
				r.second = std::max(r.second, end);
				return;
			}
		}
		dirty_ranges.emplace_back(addr, end);
	}

	int flush()
	{
		// CPU writes announced by end_write_rdram reach the device copy first, also for
		// consumers that are not passes (scanout).
		if (host_rdram_dirty)
		{
			if (check(cudaMemcpyAsync(d_rdram, host_rdram, rdram_size, cudaMemcpyHostToDevice, stream))) return sticky_error;
			host_rdram_dirty = false;
		}
		if (prims.empty() && uploads.empty())
		{
			reset_pass();
			return sticky_error;
		}
		if (coherent) collect_read_pages();

		const size_t num_recorded_prims = prims.size(), num_recorded_uploads = uploads.size();
		rdpx::PassView v = {};
		RdpPass common = {};
		common.rdram = d_rdram;
		common.hidden = d_hidden;
		common.tmem_snapshots = uploads.empty() ? d_tmem : d_snapshots;
		common.tmem_state = d_tmem;
		common.rdram_size = rdram_size;
		common.hidden_size = hidden_size;
		common.base_prim_index = uint32_t(base_prim_index);
		common.counters = d_fragments;
		common.wmask = coherent ? d_wmask : nullptr;
		// One descriptor per target; a target that does not render (no colour image, or no
		// covered line) keeps no primitives.  A pass without targets still applies its uploads.
		bool single_in_order = targets.size() == 1;
		if (targets.empty())
		{
			v.target[0] = common;
			v.target_prims[0] = 0;
			v.num_targets = 1;
		}
		for (size_t t = 0; t < targets.size(); t++)
		{
			const Target &tg = targets[t];
			bool render = tg.width != 0 && tg.deduced_height != 0 && !tg.prim_ids.empty();
			RdpPass d = common;
			d.fb_addr = tg.addr;
			d.depth_addr = tg.depth_addr;
			d.fb_width = tg.width;
			d.fb_height = std::min<uint32_t>(tg.deduced_height, RDP_MAX_TILES_Y * 8);
			d.fb_fmt = tg.fmt;
			d.tiles_x = render ? (tg.width + 7) / 8 : 0;
			d.tiles_y = render ? (d.fb_height + 7) / 8 : 0;
			v.target[t] = d;
			v.target_prims[t] = render ? uint32_t(tg.prim_ids.size()) : 0;
			if (!render) single_in_order = false;
			if (render)
			{
				add_dirty(tg.addr, tg.width * tg.deduced_height * bytes_per_pixel(tg.fmt));
				if (tg.depth_pending) add_dirty(tg.depth_addr, tg.width * tg.deduced_height * 2);
			}
		}
		if (!targets.empty()) v.num_targets = uint32_t(targets.size());
		// Primitives grouped by target (command order within a target).
		if (single_in_order)
			v.prims = prims.data();
		else
		{
			grouped.clear();
			for (size_t t = 0; t < targets.size(); t++)
				if (v.target_prims[t])
					for (uint32_t id : targets[t].prim_ids) grouped.push_back(prims[id]);
			v.prims = grouped.data();
		}
		v.num_prims = 0;
		for (uint32_t t = 0; t < v.num_targets; t++) v.num_prims += v.target_prims[t];
		v.words = words.data();
		v.num_words = uint32_t(words.size());
		v.state_blocks = state_blocks.data();
		v.num_state_blocks = uint32_t(state_blocks.size() / RDP_STATE_BLOCK_WORDS);
		v.tilesets = tilesets.data();
		v.num_tilesets = uint32_t(tilesets.size() / 8);
		v.uploads = uploads.data();
		v.num_uploads = uint32_t(uploads.size());
		v.fill_only = pass_fill_only;

		if (batch)
		{
			// The recorded buffers move into the deferred packet (reset_pass clears them anyway).
			rdpx::PassPacket pk;
			pk.targets.assign(v.target, v.target + v.num_targets);
			pk.target_prims.assign(v.target_prims, v.target_prims + v.num_targets);
			if (v.prims == prims.data() && v.num_prims == prims.size())
				pk.prims = std::move(prims);
			else
				pk.prims.assign(v.prims, v.prims + v.num_prims);
			pk.words = std::move(words);
			pk.state_blocks = std::move(state_blocks);
			pk.tilesets = std::move(tilesets);
			pk.uploads = std::move(uploads);
			if (coherent && !in_capture()) pk.read_pages = read_pages;
			pk.fill_only = v.fill_only;
			deferred.push_back(std::move(pk));
		}
		else if (up_log2)
		{
			if (coherent && refresh_pages(read_pages) != RDP_OK) return sticky_error;
			uint64_t before = exec->kernel_launches;
			if (launch_upscaled(v) != RDP_OK) return sticky_error;
			stats.kernel_launches += exec->kernel_launches - before;
		}
		else
		{
			// A capture records the GPU work only: its replays render against the device copy.
			if (coherent && !capturing && refresh_pages(read_pages) != RDP_OK) return sticky_error;
			uint64_t before = exec->kernel_launches;
			if (!exec->launch(&v, 1, capturing ? &capture_sink : nullptr)) return check(cudaErrorUnknown);
			stats.kernel_launches += exec->kernel_launches - before;
		}

		stats.passes++;
		stats.primitives += num_recorded_prims;
		stats.tmem_uploads += num_recorded_uploads;
		base_prim_index += num_recorded_prims;
		reset_pass();
		return sticky_error;
	}

	static uint32_t pixel_size_log2(uint32_t fmt)
	{
		return fmt == FBF_RGBA8888 ? 2u : (fmt == FBF_RGBA5551 || fmt == FBF_IA88) ? 1u : 0u;
	}
	// A recorded pass of an upscaling processor (Renderer::flush_queues, rdp_renderer.cpp:2953-2986).
	// Without super-sampled readback: the "pre" update of the upscaled domain over the image, the
	// 1x pass, and -- for 16/32-bit images at least 256 wide (should_render_upscaled, 2997-3009) --
	// the "post" update and the pass again at the scaled resolution (submit_render_pass 2223-2285,
	// submit_render_pass_upscaled 2287-2342).  With it: only the upscaled pass, between the "pre"
	// update plus a cleared write mask and the resolve into RDRAM.  Passes have one target here.
	int launch_upscaled(const rdpx::PassView &v)
	{
		const Target *tg = targets.empty() ? nullptr : &targets[0];
		const bool need_render_pass = tg && tg->width && tg->deduced_height && tg->span_prims;
		const uint32_t psl2 = tg ? pixel_size_log2(tg->fmt) : 0;
		const uint32_t pixels = tg ? tg->width * tg->deduced_height : 0;
		const RdpUpscaleDomain dom = up_domain();
		if (!ssaa)
		{
			if (need_render_pass && check(rdp_upscale_sync(&dom, tg->addr, tg->depth_addr, pixels, psl2, 0, stream)))
				return sticky_error;
			if (!exec->launch(&v, 1, nullptr)) return check(cudaErrorUnknown);
			if (!need_render_pass || !((tg->fmt == FBF_RGBA5551 || tg->fmt == FBF_RGBA8888) && tg->width >= 256))
				return sticky_error;
			if (check(rdp_upscale_sync(&dom, tg->addr, tg->depth_addr, pixels, psl2, 1, stream))) return sticky_error;
		}
		else
		{
			if (tg && (check(rdp_upscale_sync(&dom, tg->addr, tg->depth_addr, pixels, psl2, 0, stream)) ||
			           check(rdp_ssaa_clear_mask(&dom, tg->width, tg->deduced_height, stream))))
				return sticky_error;
			if (v.num_uploads)
			{
				// The pass's TMEM uploads (they read RDRAM itself), without its primitives.
				rdpx::PassView uv = v;
				for (uint32_t t = 0; t < uv.num_targets; t++)
				{
					uv.target_prims[t] = 0;
					uv.target[t].tiles_x = uv.target[t].tiles_y = 0;
				}
				uv.num_prims = 0;
				if (!exec->launch(&uv, 1, nullptr)) return check(cudaErrorUnknown);
			}
		}
		// The 1x launch applied the uploads; the upscaled pass samples the same TMEM snapshots.
		rdpx::PassView sv = v;
		sv.uploads = nullptr;
		sv.num_uploads = 0;
		for (uint32_t t = 0; t < sv.num_targets; t++)
		{
			RdpPass &d = sv.target[t];
			d.rdram = d_ms_rdram;
			d.hidden = d_ms_hidden;
			d.wmask = nullptr;
			d.counters = nullptr;
			d.fb_width <<= up_log2;
			d.fb_height <<= up_log2;
			d.tiles_x = sv.target_prims[t] ? (d.fb_width + 7) / 8 : 0;
			d.tiles_y = sv.target_prims[t] ? (d.fb_height + 7) / 8 : 0;
			d.scale = up_log2 | (ssaa ? 0x100u : 0u);
		}
		if (!exec->launch(&sv, 1, nullptr, true)) return check(cudaErrorUnknown);
		if (ssaa && tg &&
		    check(rdp_ssaa_resolve(&dom, tg->addr, tg->depth_addr, tg->width, tg->deduced_height, psl2, ssaa_dither, stream)))
			return sticky_error;
		return sticky_error;
	}

	void reset_pass()
	{
		prims.clear();
		words.clear();
		state_blocks.clear();
		tilesets.clear();
		uploads.clear();
		targets.clear();
		pass_fill_only = true;
		sb_dirty = true;
		tiles_dirty = true;
	}

	// A flush the reference would also perform (framebuffer change, hazard, SyncFull).
	int hard_flush()
	{
		if (ref.prims || ref.uploads) ref_pass_break();
		rv = RefView{};
		return flush();
	}

	// ================================================================= primitives
	// The target of the pass that the current colour image draws into; a new target joins
	// the pass unless the pass is full or its memory would overlap another target's.
	size_t select_target(uint32_t rows, bool uses_depth)
	{
		for (;;)
		{
			size_t ti = targets.size();
			for (size_t k = 0; k < targets.size(); k++)
			{
				const Target &t = targets[k];
				if (t.addr == fb.addr && t.width == fb.width && t.fmt == fb.fmt && t.depth_addr == fb.depth_addr)
				{
					ti = k;
					break;
				}
			}
			if (ti == targets.size())
			{
				if (targets.size() >= rdpx::kMaxTargets)
				{
					flush();
					continue;
				}
				Target t;
				t.addr = fb.addr;
				t.width = fb.width;
				t.fmt = fb.fmt;
				t.depth_addr = fb.depth_addr;
				targets.push_back(std::move(t));
			}
			if (targets.size() > 1 && target_conflicts(ti, std::max(rows, targets[ti].deduced_height), uses_depth))
			{
				flush();
				continue;
			}
			return ti;
		}
	}

	void record_prim(const uint32_t *w, uint32_t len, uint32_t op)
	{
		// A stand-alone processor hands a long pass to the GPU early when the GPU has nothing left to
		// do (the reference submits whenever no submission is active, maintain_queues,
		// rdp_renderer.cpp:2353-2371), so that the host parses on while it renders; only where the
		// pass boundary is not observable, and never while recording a capture.
		if (!batch && !capturing && !up_log2 && prims.size() >= kEagerFlushPrims &&
		    prims.size() % kEagerFlushPrims == 0 && !pass_boundaries_visible() && cudaStreamQuery(stream) == cudaSuccess)
			flush();
		if (prims.size() >= RDP_MAX_PRIMS_PER_PASS || words.size() + len > kMaxWordsPerPass ||
		    (sb_dirty && state_blocks.size() / RDP_STATE_BLOCK_WORDS >= kMaxStateBlocks) ||
		    (tiles_dirty && tilesets.size() / 8 >= kMaxTilesets))
			flush();

		// Rows the primitive reaches: the deduced framebuffer height (rdp_renderer.cpp:1556-1562).
		int yl, yh;
		bool fill_copy = cycle_type() >= 2;
		if (op >= 0x08 && op <= 0x0f)
		{
			yl = sext(w[0], 14);
			yh = sext(w[1], 14);
		}
		else
		{
			yl = int(w[0] & 0xfff);
			if (fill_copy) yl |= 3;
			yh = int(w[1] & 0xfff);
		}
		int scissor_ylo = int(sb[SB_SCISSOR] & 0xfff), scissor_yhi = int(sb[SB_SCISSOR + 1] & 0xfff);
		int max_sub = std::min(yl - 1, scissor_yhi - 1);
		uint32_t h = uint32_t(std::max((max_sub >> 2) + 1, 0));
		uint32_t om1 = sb[SB_OTHER_MODES + 1];
		bool writes_depth = (om1 & (1u << 5)) != 0;
		bool uses_depth = !fill_copy && (om1 & ((1u << 4) | (1u << 5))) != 0; // fill / copy never touch depth
		size_t ti = select_target(h, uses_depth);

		if (sb_dirty)
		{
			state_blocks.insert(state_blocks.end(), sb, sb + RDP_STATE_BLOCK_WORDS);
			sb_dirty = false;
		}
		if (tiles_dirty)
		{
			tilesets.insert(tilesets.end(), tiles, tiles + 8);
			tiles_dirty = false;
		}
		if (cycle_type() != 3) pass_fill_only = false;
		RdpPrimIn pi;
		pi.word_offset = uint32_t(words.size());
		pi.state_block = uint32_t(state_blocks.size() / RDP_STATE_BLOCK_WORDS - 1);
		pi.tileset = uint32_t(tilesets.size() / 8 - 1);
		pi.tmem_index = uint16_t(uploads.size());
		pi.seq = uint16_t(prims.size());
		prims.push_back(pi);
		words.insert(words.end(), w, w + len);

		Target &tg = targets[ti];
		tg.prim_ids.push_back(uint32_t(prims.size() - 1));
		tg.deduced_height = std::max(tg.deduced_height, h);
		tg.color_pending = true;
		tg.depth_pending |= writes_depth;
		tg.depth_used |= uses_depth;
		rv.deduced_height = std::max(rv.deduced_height, h);
		rv.color_pending = true;
		rv.depth_pending |= writes_depth;
		int min_line = std::max(yh, scissor_ylo) >> 2;
		if ((max_sub >> 2) >= min_line) tg.span_prims++;
		ref_note_prim((max_sub >> 2) - min_line + 1);

		if (validation_cb)
		{
			bool prim_depth = (om1 & (1u << 2)) != 0;
			if (cycle_type() == 3)
			{
				if (fb.fmt == FBF_I4) report(RDP_VALIDATION_FILL_4BPP, "Attempted to use Fill mode on 4bpp surface.");
				if (om1 & (1u << 4)) report(RDP_VALIDATION_FILL_DEPTH_TEST, "Attempted to use Fill mode with depth test.");
				if (om1 & (1u << 6)) report(RDP_VALIDATION_FILL_IMAGE_READ, "Attempted to use Fill mode with image read enable.");
				if ((om1 & (1u << 5)) && !prim_depth)
					report(RDP_VALIDATION_FILL_DEPTH_WRITE, "Attempted to use Fill mode with depth write enabled.");
			}
			else if (cycle_type() == 2 && fb.fmt == FBF_RGBA8888)
				report(RDP_VALIDATION_COPY_32BPP, "Attempted to use Copy mode on 32bpp surface.");
		}
		if (++rv.prims >= 256) rv_end();
	}

	// ================================================================= TMEM loads (rdp_renderer.cpp:3051-3486)
	// Does a load from `addr` read pixels of an image with writes pending (tmem_upload_needs_flush)?
	bool reads_pending(uint32_t addr, uint32_t img_addr, uint32_t width, uint32_t fmt, uint32_t depth_addr,
	                   uint32_t rows, bool color_pending, bool depth_pending) const
	{
		if (color_pending)
		{
			uint32_t offset = (addr - img_addr) & (rdram_size - 1);
			if (fmt == FBF_RGBA5551 || fmt == FBF_I8) offset >>= 1;
			else if (fmt == FBF_RGBA8888) offset >>= 2;
			if (offset < rows * width) return true;
		}
		if (depth_pending)
		{
			uint32_t offset = ((addr - depth_addr) & (rdram_size - 1)) >> 1;
			if (offset < rows * width) return true;
		}
		return false;
	}
	// The reference's hazard: its current image, writes since its own pass began.
	bool upload_needs_flush(uint32_t addr) const
	{
		return reads_pending(addr, fb.addr, fb.width, fb.fmt, fb.depth_addr, rv.deduced_height, rv.color_pending,
		                     rv.depth_pending);
	}
	// This processor's hazard: writes of any target of its (longer) pass.
	bool upload_reads_pass(uint32_t addr) const
	{
		for (const Target &t : targets)
			if (reads_pending(addr, t.addr, t.width, t.fmt, t.depth_addr, t.deduced_height, t.color_pending, t.depth_pending))
				return true;
		return false;
	}

	void load_tile(uint32_t tile, uint32_t slo, uint32_t tlo, uint32_t shi, uint32_t thi, int mode)
	{
		if (mode == 1 && (thi >> 2) > (tlo >> 2))
			report(RDP_VALIDATION_MULTILINE_TLUT, "Attempting to load multiple lines in TLUT.");
		if (upload_needs_flush(tex_image.addr)) hard_flush();
		else if (upload_reads_pass(tex_image.addr)) flush();
		if (mode != 2)
		{
			if ((thi >> 2) < (tlo >> 2)) return;
			if (!((((shi >> 2) - (slo >> 2)) + 1) & 0xfff)) return;
		}
		else
		{
			unsigned pc = ((shi - slo) + 1) & 0xfff;
			if (!pc || pc > 2048) return;
		}
		if (mode == 0)
		{
			const RdpTile &meta = tiles[tile];
			unsigned ppl = (((shi >> 2) - (slo >> 2)) + 1) & 0xfff;
			unsigned qw = ((ppl << meta.size) + 15) >> 4;
			if (meta.size > tex_image.size) qw <<= meta.size - tex_image.size;
			else if (meta.size < tex_image.size) qw >>= tex_image.size - meta.size;
			unsigned bpl = std::max<unsigned>(qw * 8, meta.stride);
			unsigned max_bpl = meta.fmt == 1 ? 0x800 : 0x1000;
			unsigned lines = ((thi >> 2) - (tlo >> 2)) + 1;
			if (bpl * lines > max_bpl)
			{
				unsigned per = (max_bpl / bpl) & ~1u;
				if (per == 0) return;
				for (unsigned line = 0; line < lines; line += per)
				{
					unsigned n = std::min(lines - line, per);
					uint32_t t_lo = tlo + (line << 2);
					load_tile_iteration(tile, slo, t_lo, shi, t_lo + ((n - 1) << 2), mode, line * meta.stride);
				}
				tiles[tile].slo = slo;
				tiles[tile].shi = shi;
				tiles[tile].tlo = tlo;
				tiles[tile].thi = thi;
				tiles_dirty = true;
				return;
			}
		}
		load_tile_iteration(tile, slo, tlo, shi, thi, mode, 0);
	}

	void load_tile_iteration(uint32_t tile, uint32_t slo, uint32_t tlo, uint32_t shi, uint32_t thi, int mode,
	                         uint32_t tmem_offset)
	{
		RdpTile &meta = tiles[tile];
		meta.slo = slo;
		meta.shi = shi;
		meta.tlo = tlo;
		meta.thi = thi;
		tiles_dirty = true;
		uint32_t isize = tex_image.size;
		if (meta.fmt == 1 && (meta.size != 2 || isize != 2)) return;
		if (isize == 0)
		{
			report(RDP_VALIDATION_LOAD_TILE_4BPP, "4-bit VRAM pointer crashes the RDP.");
			return;
		}
		if (meta.size == 3 && meta.fmt != 0) return;
		if (mode == 1 && meta.size == 3) return;
		if (mode != 1)
		{
			if (isize == 3 && meta.size == 1) return;
			if (isize == 2 && meta.size == 0) return;
			if (isize == 3 && meta.size == 0) return;
		}
		RdpUpload up = {};
		up.tmem_stride_words = int(meta.stride >> 1);
		uint32_t ux = 0, uy = 0;
		int upload_mode = mode;
		if (upload_mode == 2)
		{
			ux = slo;
			uy = tlo;
			unsigned pixel_count = (shi - slo + 1) & 0xfff;
			unsigned dt = thi;
			unsigned max_iter = (pixel_count - 1) >> (4u - isize);
			unsigned max_t = (max_iter * dt) >> 11;
			if (max_t != 0)
			{
				unsigned maxn = ((1u << 11u) + dt - 1u) / dt;
				unsigned minn = (1u << 11u) / dt;
				bool uneven = maxn != minn;
				if (uneven)
				{
					unsigned ov = (dt * maxn - (1u << 11)) * max_t;
					if (ov < dt)
					{
						minn = maxn;
						uneven = false;
					}
				}
				up.dxt = int(dt << 5);
				if (meta.size == 3 || meta.fmt == 1)
				{
					up.tmem_stride_words <<= 1;
					if (uneven && meta.size != isize) return;
				}
				if (meta.size > isize)
				{
					unsigned sh = meta.size - isize;
					maxn <<= sh;
					minn <<= sh;
					up.dxt >>= sh;
				}
				else if (isize > meta.size)
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
				upload_mode = 0;
			}
		}
		else
		{
			ux = slo >> 2;
			uy = tlo >> 2;
			up.width = int((((shi >> 2) - (slo >> 2)) + 1) & 0xfff);
			up.height = int(((thi >> 2) - (tlo >> 2)) + 1);
		}
		if (!up.width) return;
		if (isize == 1) up.vram_effective_width = (up.width + 7) & ~7;
		else if (isize == 2) up.vram_effective_width = upload_mode == 1 ? up.width : ((up.width + 3) & ~3);
		else if (isize == 3) up.vram_effective_width = (up.width + 1) & ~1;
		switch (meta.size)
		{
		case 0: up.width = ((up.width + 15) & ~15) >> 2; break;
		case 1: up.width = ((up.width + 7) & ~7) >> 1; break;
		case 2:
			up.width = (up.width + 3) & ~3;
			if (meta.fmt == 1) up.width >>= 1;
			break;
		default: up.width = (up.width + 1) & ~1; break;
		}
		if (up.height > 1 && upload_mode == 1) return;
		up.vram_addr = int(tex_image.addr + ((tex_image.width * uy + ux) << (isize - 1)));
		up.vram_width = upload_mode == 2 ? up.vram_effective_width : int(tex_image.width);
		up.vram_size = int(isize);
		up.tmem_offset = int((meta.offset + tmem_offset) & 0xfff);
		up.tmem_size = meta.size;
		up.tmem_fmt = meta.fmt;
		up.mode = upload_mode;
		up.inv_tmem_stride_words = 1.0f / float(up.tmem_stride_words);
		uploads.push_back(up);
		ref.uploads++;
		if (ref.uploads + 1 >= 256) ref_pass_break();
		if (++rv.uploads + 1 >= 256) rv_end();
		if (uploads.size() + 1 >= RDP_MAX_UPLOADS_PER_PASS) flush();
	}

	// ================================================================= command dispatch
	void set_tile(const uint32_t *w)
	{
		RdpTile &t = tiles[(w[1] >> 24) & 7];
		t.offset = ((w[0] >> 0) & 511) << 3;
		t.stride = ((w[0] >> 9) & 511) << 3;
		t.size = uint8_t((w[0] >> 19) & 3);
		t.fmt = uint8_t((w[0] >> 21) & 7);
		t.palette = uint8_t((w[1] >> 20) & 15);
		t.shift_s = uint8_t((w[1] >> 0) & 15);
		t.mask_s = uint8_t((w[1] >> 4) & 15);
		t.shift_t = uint8_t((w[1] >> 10) & 15);
		t.mask_t = uint8_t((w[1] >> 14) & 15);
		t.flags = 0;
		if (w[1] & (1u << 8)) t.flags |= TIF_MIRROR_S;
		if (w[1] & (1u << 9)) t.flags |= TIF_CLAMP_S;
		if (w[1] & (1u << 18)) t.flags |= TIF_MIRROR_T;
		if (w[1] & (1u << 19)) t.flags |= TIF_CLAMP_T;
		if (t.mask_s > 10) t.mask_s = 10;
		else if (t.mask_s == 0) t.flags |= TIF_CLAMP_S;
		if (t.mask_t > 10) t.mask_t = 10;
		else if (t.mask_t == 0) t.flags |= TIF_CLAMP_T;
		tiles_dirty = true;
	}

	void set_state(int index, const uint32_t *w)
	{
		if (sb[index] != w[0] || sb[index + 1] != w[1])
		{
			sb[index] = w[0];
			sb[index + 1] = w[1];
			sb_dirty = true;
		}
	}

	void command(const uint32_t *w)
	{
		uint32_t op = (w[0] >> 24) & 63;
		switch (op)
		{
		case 0x01: // MetaSignalTimeline (rdp_device.cpp:926-934): words 1-2 are the value
			signal_value(uint64_t(w[1]) | (uint64_t(w[2]) << 32));
			break;
		case 0x02: // MetaFlush (rdp_device.cpp:936-940)
			hard_flush();
			break;
		case 0x03: // MetaIdle (rdp_device.cpp:942-946): a hint that the command stream went quiet;
			break;  // this processor submits at flushes and timeline values, so nothing is pending
		case 0x04: // MetaSetQuirks (rdp_device.cpp:948-952)
			if (sb[SB_QUIRKS] != w[1]) { sb[SB_QUIRKS] = w[1]; sb_dirty = true; }
			break;
		case 0x08: case 0x09: case 0x0a: case 0x0b: case 0x0c: case 0x0d: case 0x0e: case 0x0f:
		case 0x24: case 0x25: case 0x36:
			record_prim(w, command_length(op), op);
			break;
		case 0x29: hard_flush(); break;
		case 0x2a: set_state(SB_KEY_GB, w); break;
		case 0x2b: set_state(SB_KEY_R, w); break;
		case 0x2c: set_state(SB_CONVERT, w); break;
		case 0x2d: set_state(SB_SCISSOR, w); break;
		case 0x2e: set_state(SB_PRIM_DEPTH, w); break;
		case 0x2f: set_state(SB_OTHER_MODES, w); break;
		case 0x30: load_tile((w[1] >> 24) & 7, (w[0] >> 12) & 0xfff, w[0] & 0xfff, (w[1] >> 12) & 0xfff, w[1] & 0xfff, 1); break;
		case 0x32:
		{
			RdpTile &t = tiles[(w[1] >> 24) & 7];
			t.slo = (w[0] >> 12) & 0xfff;
			t.shi = (w[1] >> 12) & 0xfff;
			t.tlo = w[0] & 0xfff;
			t.thi = w[1] & 0xfff;
			tiles_dirty = true;
			break;
		}
		case 0x33: load_tile((w[1] >> 24) & 7, (w[0] >> 12) & 0xfff, w[0] & 0xfff, (w[1] >> 12) & 0xfff, w[1] & 0xfff, 2); break;
		case 0x34: load_tile((w[1] >> 24) & 7, (w[0] >> 12) & 0xfff, w[0] & 0xfff, (w[1] >> 12) & 0xfff, w[1] & 0xfff, 0); break;
		case 0x35: set_tile(w); break;
		case 0x37: set_state(SB_FILL_COLOR, w); break;
		case 0x38: set_state(SB_FOG_COLOR, w); break;
		case 0x39: set_state(SB_BLEND_COLOR, w); break;
		case 0x3a: set_state(SB_PRIM_COLOR, w); break;
		case 0x3b: set_state(SB_ENV_COLOR, w); break;
		case 0x3c: set_state(SB_COMBINE, w); break;
		case 0x3d:
			tex_image.fmt = (w[0] >> 21) & 7;
			tex_image.size = (w[0] >> 19) & 3;
			tex_image.width = (w[0] & 0x3ff) + 1;
			tex_image.addr = w[1] & 0xffffff;
			break;
		case 0x3e:
		{
			uint32_t a = w[1] & 0xffffff;
			if (a != fb.depth_addr) hard_flush();
			fb.depth_addr = a;
			break;
		}
		case 0x3f:
		{
			uint32_t f = (w[0] >> 21) & 7, size = (w[0] >> 19) & 3;
			uint32_t width = (w[0] & 1023) + 1, addr = w[1] & 0xffffff;
			uint32_t fmt = size == 0 ? FBF_I4 : size == 1 ? FBF_I8 : size == 2 ? (f ? FBF_IA88 : FBF_RGBA5551) : FBF_RGBA8888;
			if (addr != fb.addr || width != fb.width || fmt != fb.fmt)
			{
				// The reference ends its pass here.  This processor keeps the pass open (the new
				// image becomes another target) unless either image has visible pass boundaries.
				if (!pass_boundaries_visible() && !boundaries_visible(fmt, addr, fb.depth_addr))
				{
					if (ref.prims || ref.uploads) ref_pass_break();
					rv = RefView{};
				}
				else
					hard_flush();
			}
			fb.addr = addr;
			fb.width = width;
			fb.fmt = fmt;
			break;
		}
		default:
			break;
		}
	}

	int enqueue(uint32_t n, const uint32_t *w)
	{
		uint32_t i = 0;
		if (!carry.empty())
		{
			uint32_t need = command_length((carry[0] >> 24) & 63);
			while (carry.size() < need && i < n) carry.push_back(w[i++]);
			if (carry.size() < need) return sticky_error;
			command(carry.data());
			carry.clear();
		}
		while (i < n)
		{
			uint32_t len = command_length((w[i] >> 24) & 63);
			if (i + len > n)
			{
				carry.assign(w + i, w + n);
				break;
			}
			command(w + i);
			i += len;
		}
		return sticky_error;
	}


	// ================================================================= Video Interface
	struct ViRegs
	{
		int vi_width, vi_offset, v_current_line, v_start, init_y_add, v_res, is_pal, max_x, max_y;
		int h_start, h_res, h_start_clamp, h_res_clamp;
		uint32_t status;
	};

	// decode_vi_registers (video_interface.cpp:177-367).
	ViRegs vi_decode(RdpViLine *lines)
	{
		const uint32_t *R = vi_regs;
		ViRegs r = {};
		r.status = R[0];
		r.vi_width = R[2] & 0xfff;
		r.vi_offset = R[1] & 0xffffff;
		r.v_current_line = R[4] & 1;
		r.v_start = (R[10] >> 16) & 0x3ff;
		int y_start = (R[13] >> 16) & 0xfff, y_add = R[13] & 0xfff;
		r.init_y_add = y_add;
		int v_end = R[10] & 0x3ff, v_sync = R[6] & 0x3ff;
		r.is_pal = unsigned(v_sync) > 525u + 25u;
		const int v_end_max = r.is_pal ? ((44 + 576) | 1) : ((34 + 480) | 1);
		if (v_end > v_end_max) v_end = v_end_max;
		if (r.v_start > v_end_max) r.v_start = v_end_max;
		int v_start_offset = r.is_pal ? 44 : 34;
		r.v_res = (v_end - r.v_start) >> 1;
		r.v_start = (r.v_start - v_start_offset) / 2;
		if (r.v_start < 0)
		{
			y_start -= y_add * r.v_start;
			r.v_start = 0;
		}
		r.v_res = std::min(r.v_res, RDP_VI_MAX_LINES - r.v_start);
		int hsc_lo = INT32_MAX, hec_hi = 0, hs_lo = INT32_MAX, he_hi = 0;
		r.max_x = 0;
		bool degenerate_y = r.v_res <= 0;
		for (int i = 0; i < RDP_VI_MAX_LINES; i++)
			if (degenerate_y || i < r.v_start || i >= r.v_start + r.v_res) lines[i] = RdpViLine{};
		const int h_offset = r.is_pal ? 128 : 108;
		auto analyze = [&](int x_start, int x_add, int h_start, int h_end, RdpViLine *line) {
			bool lc = false, rc = false;
			h_start -= h_offset;
			h_end -= h_offset;
			if (h_start < 0)
			{
				x_start -= x_add * h_start;
				h_start = 0;
				lc = true;
			}
			if (h_end > 640)
			{
				h_end = 640;
				rc = true;
			}
			int hsc = h_start + (lc ? 0 : 8), hec = h_end - (rc ? 0 : 7);
			int h_res = h_end - h_start;
			r.max_x = std::max(r.max_x, (x_start + h_res * x_add) >> 10);
			hs_lo = std::min(hs_lo, h_start);
			he_hi = std::max(he_hi, h_end);
			hsc_lo = std::min(hsc_lo, hsc);
			hec_hi = std::max(hec_hi, hec);
			if (line) *line = RdpViLine{ h_start, hsc, hec, x_start, x_add, y_start, y_add, 0 };
		};
		if (degenerate_y || !vi.ended)
		{
			RdpViLine li;
			analyze((R[12] >> 16) & 0xfff, R[12] & 0xfff, (R[9] >> 16) & 0x3ff, R[9] & 0x3ff, &li);
			for (int i = r.v_start; i < r.v_start + r.v_res; i++) lines[i] = li;
		}
		else
		{
			for (int i = r.v_start; i < r.v_start + r.v_res; i++)
			{
				int eff = 2 * i + v_start_offset + int(r.v_current_line == 0);
				analyze((vi.xs_line[eff] >> 16) & 0xfff, vi.xs_line[eff] & 0xfff, (vi.hs_line[eff] >> 16) & 0x3ff,
				        vi.hs_line[eff] & 0x3ff, &lines[i]);
			}
		}
		r.max_y = (y_start + r.v_res * y_add) >> 10;
		r.h_start = hs_lo;
		r.h_res = he_hi - hs_lo;
		r.h_start_clamp = hsc_lo;
		r.h_res_clamp = hec_hi - hsc_lo;
		return r;
	}

	// VideoInterface::scanout_memory_range (video_interface.cpp:369-396): the bytes the fetch reads,
	// from the registers with the per-scanline state cleared (as scanout leaves it).
	void vi_memory_range(uint32_t &off, uint32_t &len)
	{
		RdpViLine tmp[RDP_VI_MAX_LINES];
		const bool ended = vi.ended;
		vi.ended = false;
		const ViRegs m = vi_decode(tmp);
		vi.ended = ended;
		const bool dv = (m.status & (1u << 4)) != 0;
		const int aw = m.max_x + 2 + 4 + int(dv) * 2, ah = m.max_y + 1 + 4;
		if (m.vi_offset == 0 || m.h_res <= 0 || m.h_start >= 640)
		{
			off = len = 0;
			return;
		}
		const int ps = (((m.status & 3u) | 2u) == 3u) ? 4 : 2;
		off = uint32_t((m.vi_offset & ~(ps - 1)) + ((dv ? -3 : -2) - 2 * m.vi_width) * ps);
		len = uint32_t((ah * m.vi_width + aw) * ps);
	}

	int vi_ensure(uint32_t **buf, size_t *cap, size_t words)
	{
		if (*cap >= words) return RDP_OK;
		cudaStreamSynchronize(stream);
		cudaFree(*buf);
		*buf = nullptr;
		*cap = 0;
		if (check(cudaMalloc(buf, words * 4))) return RDP_ERR_OOM;
		*cap = words;
		return RDP_OK;
	}

	// VideoInterface::scanout (video_interface.cpp:1215-1426) at 1x scale, into `out` (host).
	int scanout(const rdp_scanout_options *o, uint32_t *out, uint32_t *width, uint32_t *height)
	{
		const uint32_t *img = nullptr;
		int r = scanout_device(o, &img, width, height);
		if (r != RDP_OK || !img) return r;
		if (check(cudaMemcpyAsync(out, img, size_t(*width) * *height * 4, cudaMemcpyDeviceToHost, stream))) return sticky_error;
		return check(cudaStreamSynchronize(stream));
	}

	// The scanout image in device memory (*img = nullptr: no image).  The VI kernels are queued on
	// the processor's stream; the image is one of two that alternate (the other is the previous
	// frame, which the next scanout may blend with).
	int scanout_device(const rdp_scanout_options *o, const uint32_t **img, uint32_t *width, uint32_t *height)
	{
		*img = nullptr;
		*width = *height = 0;
		int r0 = sync_point();
		if (r0 != RDP_OK) return r0;
		if (!vi.tables)
		{
			if (check(rdp_vi_init_tables())) return sticky_error;
			if (check(cudaMalloc(&vi.d_lines, sizeof(RdpViLine) * RDP_VI_MAX_LINES))) return RDP_ERR_OOM;
			for (auto &b : vi.d_out)
				if (check(cudaMalloc(&b, (size_t(640) * 576 * 4) << (2 * up_log2)))) return RDP_ERR_OOM;
			vi.tables = true;
		}
		RdpViLine lines[RDP_VI_MAX_LINES];
		ViRegs r = vi_decode(lines);
		vi.flags = 0;
		vi.ended = false;
		if (r.vi_offset == 0)
		{
			vi.have_prev = false;
			return RDP_OK;
		}
		if (!o->vi_serrate) r.status &= ~(1u << 6);
		bool is_aa = (r.status & (3u << 8)) < (2u << 8) && o->vi_aa;
		bool is_bilinear = (r.status & (3u << 8)) < (3u << 8) && o->vi_scale;
		r.status &= ~((3u << 8) | (1u << 17) | (1u << 18));
		if (is_aa) r.status |= 1u << 17;
		if (is_bilinear) r.status |= 1u << 18;
		if (!o->vi_gamma_dither) r.status &= ~(1u << 2);
		if (!o->vi_divot_filter) r.status &= ~(1u << 4);
		if (!o->vi_dither_filter) r.status &= ~(1u << 16);
		bool is_blank = (r.status & 2u) == 0;
		if (is_blank && vi.previous_frame_blank)
		{
			vi.frame_count++;
			vi.have_prev = false;
			return RDP_OK;
		}
		if (is_blank) vi.have_prev = false;
		r.status |= 2u;
		vi.previous_frame_blank = is_blank;
		bool divot = (r.status & (1u << 4)) != 0;
		if (r.h_res <= 0 || r.h_start >= 640)
		{
			vi.frame_count++;
			if (o->persist_frame_on_invalid_input && (vi.frame_count - vi.last_valid_frame_count < 4) && vi.have_prev)
			{
				*width = uint32_t(vi.prev_w);
				*height = uint32_t(vi.prev_h);
				*img = vi.d_out[vi.cur ^ 1];
				return RDP_OK;
			}
			vi.have_prev = false;
			return RDP_OK;
		}
		vi.last_valid_frame_count = vi.frame_count;
		bool degenerate = r.h_res <= 0 || r.v_res <= 0;
		bool is_8888 = (r.status & 3u) == 3u;
		const int native_max_y = r.max_y;
		// Upscaled scanout works in scaled pixels (video_interface.cpp:1299-1318).
		const int S = 1 << up_log2;
		if (up_log2)
		{
			r.h_start *= S;
			r.h_start_clamp *= S;
			r.v_start *= S;
			r.h_res *= S;
			r.h_res_clamp *= S;
			r.v_res *= S;
			r.max_x = r.max_x * S + (S - 1);
			r.max_y = r.max_y * S + (S - 1);
			for (RdpViLine &li : lines)
			{
				li.h_start *= S;
				li.h_start_clamp *= S;
				li.h_end_clamp *= S;
				li.x_start *= S;
				li.y_start *= S;
				li.y_base *= S;
			}
		}

		RdpViParams p = {};
		p.rdram = up_log2 ? d_ms_rdram : d_rdram;
		p.hidden = up_log2 ? d_ms_hidden : d_hidden;
		p.rdram_size = rdram_size;
		p.scale_log2 = int(up_log2);
		p.fb_offset = is_8888 ? (r.vi_offset >> 2) : (r.vi_offset >> 1);
		p.fb_width = r.vi_width;
		p.is_8888 = is_8888;
		p.fetch_aa = (r.status & (1u << 17)) != 0;
		p.dither_filter = (r.status & (1u << 16)) != 0;
		p.divot = divot;
		p.fetch_bug = r.init_y_add < 1024 && !up_log2; // need_fetch_bug_emulation (video_interface.cpp:398-403)
		p.degenerate = degenerate;
		if (!degenerate)
		{
			p.aa_w = r.max_x + 3 + int(divot) * 2;
			p.aa_h = r.max_y + 2;
			if (vi_ensure(&vi.d_aa, &vi.aa_cap, size_t(p.aa_w) * p.aa_h * 2) != RDP_OK) return RDP_ERR_OOM;
			p.aa = vi.d_aa;
			if (divot)
			{
				p.dv_w = r.max_x + 2;
				p.dv_h = r.max_y + 2;
				if (vi_ensure(&vi.d_dv, &vi.dv_cap, size_t(p.dv_w) * p.dv_h * 2) != RDP_OK) return RDP_ERR_OOM;
				p.dv = vi.d_dv;
			}
			else
			{
				p.dv = p.aa;
				p.dv_w = p.aa_w;
				p.dv_h = p.aa_h;
			}
		}

		bool serrate = (r.status & (1u << 6)) != 0 && !o->upscale_deinterlacing;
		int w = 640 * S, h = ((r.is_pal ? 576 : 480) >> int(!serrate)) * S;
		unsigned cl, cr, ct, cb;
		if (o->crop_rect_enable)
		{
			cl = o->crop_left; cr = o->crop_right; ct = o->crop_top; cb = o->crop_bottom;
			if (serrate) { ct *= 2; cb *= 2; }
		}
		else
		{
			unsigned cy = o->crop_overscan_pixels * (serrate ? 2 : 1);
			unsigned cx = unsigned(std::round(float(cy) * (float(w) / float(h))));
			cl = cr = cx;
			ct = cb = cy;
		}
		cl *= unsigned(S);
		cr *= unsigned(S);
		ct *= unsigned(S);
		cb *= unsigned(S);
		if (cl + cr < unsigned(w) && ct + cb < unsigned(h))
		{
			w -= int(cl + cr);
			h -= int(ct + cb);
		}
		p.lines = vi.d_lines;
		p.out = vi.d_out[vi.cur];
		p.out_w = w;
		p.out_h = h;
		p.prev = vi.d_out[vi.cur ^ 1];
		p.prev_w = vi.prev_w;
		p.prev_h = vi.prev_h;
		p.crop_left = int(cl);
		p.crop_top = int(ct);
		p.v_start = r.v_start;
		p.v_res = r.v_res;
		p.info_y_shift = int(up_log2);
		if (serrate)
		{
			p.v_start *= 2;
			p.v_res *= 2;
			p.serrate_shift = 1;
			p.serrate_mask = 1;
			p.serrate_select = int(r.v_current_line == 0);
			p.info_y_shift++;
		}
		p.h_start = r.h_start;
		p.h_res = r.h_res;
		p.h_start_clamp = r.h_start_clamp;
		p.h_res_clamp = r.h_res_clamp;
		p.draw = !degenerate && r.h_res > 0 && r.v_res > 0;
		p.init_y_add = r.init_y_add;
		p.frame_count = vi.frame_count;
		p.scale_aa = (r.status & (1u << 18)) != 0;
		p.gamma = (r.status & (1u << 3)) != 0;
		p.gamma_dither = (r.status & (1u << 2)) != 0;
		p.blend_prev = vi.have_prev && o->blend_previous_frame;
		if (coherent && !degenerate)
		{
			// The VI reads the framebuffer lines it scans: those pages come from the caller's RDRAM
			// first (resolve_coherency_external, rdp_device.cpp:1103).
			begin_page_list();
			mark_read_range(r.vi_offset, uint64_t(std::max(r.vi_width, 1)) * uint64_t(std::max(native_max_y, 0) + 3) *
			                                 (is_8888 ? 4u : 2u));
			if (refresh_all) mark_read_range(0, rdram_size);
			refresh_all = false;
			if (refresh_pages(read_pages) != RDP_OK) return sticky_error;
		}
		// The per-line registers are copied from pinned memory that the next scanout rewrites only
		// after this copy has finished.
		if (vi.lines_copied && check(cudaEventSynchronize(vi.lines_copied))) return sticky_error;
		if (!vi.h_lines)
		{
			if (check(cudaMallocHost(&vi.h_lines, sizeof(lines)))) return RDP_ERR_OOM;
			if (check(cudaEventCreateWithFlags(&vi.lines_copied, cudaEventDisableTiming))) return sticky_error;
		}
		memcpy(vi.h_lines, lines, sizeof(lines));
		if (check(cudaMemcpyAsync(vi.d_lines, vi.h_lines, sizeof(lines), cudaMemcpyHostToDevice, stream))) return sticky_error;
		if (check(cudaEventRecord(vi.lines_copied, stream))) return sticky_error;
		if (up_log2 && !degenerate)
		{
			// The fetch first brings the scanned range of the upscaled domain up to date with RDRAM
			// (VideoInterface::vram_fetch_stage, video_interface.cpp:410-420).
			uint32_t off, len;
			vi_memory_range(off, len);
			const RdpUpscaleDomain dom = up_domain();
			if (check(rdp_upscale_sync(&dom, off, off, len, is_8888 ? 2u : 1u, 0, stream))) return sticky_error;
		}
		if (check(rdp_vi_launch(&p, stream))) return sticky_error;
		// downscale_stage (video_interface.cpp:1000-1064): halve while the factor allows.
		for (uint32_t steps = std::min(8u, o->downscale_steps), f = uint32_t(S); f > 1 && steps; f >>= 1, steps--)
		{
			if (vi_ensure(&vi.d_half, &vi.half_cap, size_t(w / 2) * size_t(h / 2)) != RDP_OK) return RDP_ERR_OOM;
			if (check(rdp_vi_downscale(p.out, w, h, vi.d_half, stream))) return sticky_error;
			w /= 2;
			h /= 2;
			if (check(cudaMemcpyAsync(p.out, vi.d_half, size_t(w) * h * 4, cudaMemcpyDeviceToDevice, stream)))
				return sticky_error;
		}
		*img = p.out;
		*width = uint32_t(w);
		*height = uint32_t(h);
		vi.prev_w = w;
		vi.prev_h = h;
		vi.have_prev = true;
		vi.cur ^= 1;
		vi.frame_count++;
		return RDP_OK;
	}

	void vi_begin_per_scanline(uint32_t flags)
	{
		vi.flags = flags;
		vi.hs_latched = vi_regs[9];
		vi.xs_latched = vi_regs[12];
		vi.hs_line[0] = vi_regs[9];
		vi.xs_line[0] = vi_regs[12];
		vi.line = 0;
		vi.ended = false;
	}
	void vi_set_for_scanline(uint32_t reg, uint32_t value)
	{
		if ((vi.flags & reg) == 0) return;
		if (reg == 1) vi.hs_latched = value;
		else if (reg == 2) vi.xs_latched = value;
	}
	void vi_latch_scanline(unsigned line)
	{
		const unsigned v_end_max = (44 + 576) | 1;
		line = std::min(line, v_end_max - 1);
		if (line <= vi.line) return;
		unsigned c = vi.line;
		while (++c < line)
		{
			vi.hs_line[c] = vi.hs_line[vi.line];
			vi.xs_line[c] = vi.xs_line[vi.line];
		}
		vi.hs_line[c] = vi.hs_latched;
		vi.xs_line[c] = vi.xs_latched;
		vi.line = c;
	}
	void vi_end_per_scanline()
	{
		const unsigned v_end_max = (44 + 576) | 1;
		if (vi.flags == 0 || vi.ended) return;
		unsigned c = vi.line;
		while (++c < v_end_max)
		{
			vi.hs_line[c] = vi.hs_line[vi.line];
			vi.xs_line[c] = vi.xs_line[vi.line];
		}
		vi.ended = true;
	}

	// ================================================================= timeline + coherency
	cudaEvent_t get_event()
	{
		if (!free_events.empty())
		{
			cudaEvent_t e = free_events.back();
			free_events.pop_back();
			return e;
		}
		cudaEvent_t e = nullptr;
		cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
		return e;
	}

	int copy_back()
	{
		if (coherent)
		{
			CohLauncher cl;
			cl.begin(stream, 1);
			write_back_pages(cl);
			return check(cl.finish(stream, 1));
		}
		for (auto &r : dirty_ranges)
		{
			if (host_registered)
			{
				if (check(cudaMemcpyAsync(host_rdram + r.first, d_rdram + r.first, r.second - r.first,
				                          cudaMemcpyDeviceToHost, stream)))
					return sticky_error;
			}
			else
			{
				if (check(cudaStreamSynchronize(stream))) return sticky_error;
				if (check(cudaMemcpy(host_rdram + r.first, d_rdram + r.first, r.second - r.first,
				                     cudaMemcpyDeviceToHost)))
					return sticky_error;
			}
		}
		dirty_ranges.clear();
		return sticky_error;
	}

	int batch_submit(); // defined after rdp_batch

	// A batched instance's deferred passes have been launched (rdp_batch::submit): its
	// signalled timeline values complete after them and after the copy-back.
	int complete_submitted(CohLauncher *write_back)
	{
		if (unsubmitted.empty()) return sticky_error;
		if (coherent && write_back) write_back_pages(*write_back); // launched by the caller, for all instances
		else if (copy_back() != RDP_OK) return sticky_error;
		for (uint64_t v : unsubmitted)
		{
			cudaEvent_t e = get_event();
			if (!e) return RDP_ERR_DEVICE;
			if (check(cudaEventRecord(e, stream))) return sticky_error;
			pending.emplace_back(v, e);
		}
		unsubmitted.clear();
		return sticky_error;
	}

	// Work that must be on the stream before the caller reads device state.
	int sync_point()
	{
		int r = hard_flush();
		if (r != RDP_OK || !batch) return r;
		return batch_submit();
	}

	int signal_timeline(uint64_t *value)
	{
		const uint64_t v = timeline_counter + 1;
		int r = signal_value(v);
		if (value) *value = v;
		return r;
	}

	// Everything recorded so far completes with timeline value v (values only grow: a value not
	// above the current one completes together with it).
	int signal_value(uint64_t v)
	{
		if (hard_flush() != RDP_OK) return sticky_error;
		v = std::max(v, timeline_counter);
		timeline_counter = v;
		if (batch)
		{
			unsubmitted.push_back(v);
			return sticky_error;
		}
		if (copy_back() != RDP_OK) return sticky_error;
		{
			std::lock_guard<std::mutex> hold(timeline_mu);
			cudaEvent_t e = get_event();
			if (!e) return RDP_ERR_DEVICE;
			if (check(cudaEventRecord(e, stream))) return sticky_error;
			pending.emplace_back(v, e);
		}
		decoded_value.store(v);
		return RDP_OK;
	}

	// Completion query for `value` that never launches deferred work (unlike wait_timeline,
	// which submits the batch when `value` still waits for it): RDP_ERR_TIMEOUT while pending.
	int poll_timeline(uint64_t value)
	{
		if (batch && !unsubmitted.empty() && unsubmitted.front() <= value) return RDP_ERR_TIMEOUT;
		return wait_timeline(value, 0);
	}

	int wait_timeline(uint64_t value, uint64_t timeout_ns)
	{
		// Timeouts beyond ~11 days mean "no deadline" (and must not overflow the clock).
		if (batch && !unsubmitted.empty() && unsubmitted.front() <= value)
		{
			int r = batch_submit();
			if (r != RDP_OK) return r;
		}
		const bool bounded = timeout_ns < (uint64_t(1) << 50);
		auto deadline = std::chrono::steady_clock::now() + std::chrono::nanoseconds(bounded ? int64_t(timeout_ns) : 0);
		if (ring)
		{
			// The worker must first have decoded the value's MetaSignalTimeline.  A value above the
			// ones handed out here can only come in band: once everything pushed is decoded (the
			// worker then waits, so its counter can be read), it is known or never signalled.
			if (value > api_value)
			{
				ring->drain();
				if (value > timeline_counter) return RDP_ERR_INVALID;
			}
			else if (!ring->wait_until([&] { return decoded_value.load() >= value; }, deadline, bounded))
				return RDP_ERR_TIMEOUT;
		}
		// Values complete in order; `value` has completed once a value at or above it has (a value
		// signalled in band may be larger than the caller's own next one).
		std::unique_lock<std::mutex> hold(timeline_mu);
		while (!pending.empty() && completed_value < value)
		{
			cudaEvent_t e = pending.front().second;
			for (;;)
			{
				cudaError_t q = cudaEventQuery(e);
				if (q == cudaSuccess) break;
				if (q != cudaErrorNotReady) return check(q);
				if (bounded && std::chrono::steady_clock::now() >= deadline) return RDP_ERR_TIMEOUT;
				hold.unlock();
				std::this_thread::yield();
				hold.lock();
				if (pending.empty() || pending.front().second != e) break; // another waiter took it
			}
			if (pending.empty() || pending.front().second != e) continue;
			completed_value = pending.front().first;
			free_events.push_back(e);
			pending.pop_front();
		}
		if (!ring && value > timeline_counter) return RDP_ERR_INVALID;
		return sticky_error;
	}

	int idle()
	{
		if (ring)
		{
			uint64_t v = 0;
			int r = api_signal(&v);
			if (r == RDP_OK) r = wait_timeline(v, UINT64_MAX / 2);
			if (r == RDP_OK) own_exec.tune_epoch();
			return r;
		}
		uint64_t v = 0;
		int r = signal_timeline(&v);
		if (r != RDP_OK) return r;
		r = wait_timeline(v, UINT64_MAX / 2);
		if (r == RDP_OK && !batch)
		{
			own_exec.tune_epoch();
			r = device_error_status(own_exec);
		}
		return r;
	}

	// A bounded wait inside a kernel gave up: the results of the work since the last check are
	// incomplete.  Reported, and sticky.
	int device_error_status(rdpx::Executor &ex)
	{
		const uint32_t e = ex.take_device_error();
		if (!e) return sticky_error;
		report(-1, "a bounded wait on the GPU gave up; the work since the last timeline value is incomplete");
		sticky_error = RDP_ERR_TIMEOUT;
		return sticky_error;
	}

	// ---------------------------------------------------------------- C ABI side of the command thread
	// Without a command thread these decode on the calling thread.
	int api_enqueue(uint32_t n, const uint32_t *w)
	{
		if (!ring) return enqueue(n, w);
		ring->push(n, w);
		return sticky_error;
	}
	int api_signal(uint64_t *value)
	{
		if (!ring) return signal_timeline(value);
		const uint64_t v = ++api_value;
		const uint32_t w[3] = { 0x01u << 24, uint32_t(v), uint32_t(v >> 32) };
		ring->push(3, w);
		if (value) *value = v;
		return sticky_error;
	}
	int api_flush()
	{
		if (!ring) return hard_flush();
		const uint32_t w[1] = { 0x02u << 24 };
		ring->push(1, w);
		return sticky_error;
	}
	// Before the caller touches decoder or device state directly: every pushed word is decoded
	// and the worker waits for more.
	void sync_ring()
	{
		if (ring) ring->drain();
	}
	int start_command_thread()
	{
		ring = new (std::nothrow) CommandRing();
		if (!ring) return RDP_ERR_OOM;
		ring->start([this](uint32_t n, const uint32_t *w) {
			cudaSetDevice(device);
			enqueue(n, w);
		});
		return RDP_OK;
	}
	void stop_command_thread()
	{
		if (!ring) return;
		ring->drain();
		ring->stop();
		delete ring;
		ring = nullptr;
	}
};

// ============================================================================ batch
// Many instances, one executor: each round launches the next deferred pass of every
// instance that has one, so one kernel chain renders all instances' passes together.
struct rdp_batch
{
	int device = 0;
	uint32_t flags = 0;
	cudaStream_t stream = nullptr;
	rdpx::Executor exec;
	std::vector<rdp_cp *> instances;
	bool capturing = false;
	rdpx::CaptureSink sink;
	uint64_t rounds = 0, passes = 0;
	int sticky_error = RDP_OK;
	// Host threads that parse many instances' command words at once (rdp_batch_enqueue_many,
	// the serving loop's admissions).  A task owns one instance, and run() returns only once
	// every task has finished, so no instance's recorder is ever touched by two threads, and
	// nothing reads the recorders (submit, completion polls) while a parse is running.
	rdpx::HostPool parse_pool;

	bool reserve_for_capture();

	int submit()
	{
		if (sticky_error != RDP_OK) return sticky_error;
		exec.tune_collect();
		std::vector<rdpx::PassView> views;
		std::vector<rdp_cp *> owners;
		views.reserve(instances.size());
		owners.reserve(instances.size());
		if (capturing && !reserve_for_capture()) return sticky_error = RDP_ERR_DEVICE;
		// Every page the submitted passes read comes from the callers' RDRAM first, in one launch for
		// all instances and rounds (each page once per instance).  Refreshing a later round's pages
		// before the earlier rounds run is the same as refreshing them just before their round: the
		// caller's writes all precede the submission, and bytes the earlier rounds write set the mask
		// after the refresh, so they stay the GPU's.
		{
			CohLauncher refresh;
			refresh.begin(stream, 0);
			for (rdp_cp *cp : instances)
			{
				if (cp->deferred.empty() || !cp->coherent) continue;
				cp->begin_page_list();
				for (const rdpx::PassPacket &pk : cp->deferred)
					for (uint32_t pg : pk.read_pages)
						if (cp->page_stamp[pg] != cp->stamp)
						{
							cp->page_stamp[pg] = cp->stamp;
							refresh.add(cp->host_mapped, cp->d_rdram, cp->d_wmask, pg);
						}
			}
			if (refresh.finish(stream, 0) != cudaSuccess) return sticky_error = RDP_ERR_DEVICE;
		}
		for (;;)
		{
			views.clear();
			owners.clear();
			for (rdp_cp *cp : instances)
				if (!cp->deferred.empty())
				{
					views.push_back(cp->deferred.front().view());
					owners.push_back(cp);
				}
			if (views.empty()) break;
			if (!exec.launch(views.data(), uint32_t(views.size()), capturing ? &sink : nullptr))
				return sticky_error = RDP_ERR_DEVICE;
			rounds++;
			passes += views.size();
			for (rdp_cp *cp : owners) cp->deferred.pop_front();
		}
		// Masked write-back of every signalled instance's pages in as few launches as possible, then
		// the instances' timeline events after it.
		CohLauncher write_back;
		write_back.begin(stream, 1);
		std::vector<rdp_cp *> signalled;
		for (rdp_cp *cp : instances)
			if (!cp->unsubmitted.empty())
			{
				signalled.push_back(cp);
				if (cp->coherent) cp->write_back_pages(write_back);
			}
		if (write_back.finish(stream, 1) != cudaSuccess) return sticky_error = RDP_ERR_DEVICE;
		for (rdp_cp *cp : signalled)
		{
			int r = cp->complete_submitted(nullptr);
			if (r != RDP_OK) return sticky_error = r;
		}
		return RDP_OK;
	}
};

int rdp_cp::batch_submit() { return batch->submit(); }
bool rdp_cp::in_capture() const { return capturing || (batch && batch->capturing); }

// Recorded launches keep pointers to the executor's buffers, so the buffers are sized for
// every round of a capture before the first one is recorded.
bool rdp_batch::reserve_for_capture()
{
	rdpx::ExecCaps need = exec.caps;
	size_t depth = 0;
	for (rdp_cp *cp : instances) depth = std::max(depth, cp->deferred.size());
	std::vector<rdpx::PassView> views;
	for (size_t r = 0; r < depth; r++)
	{
		views.clear();
		uint32_t prims = 0, tiles = 0, uploads = 0;
		size_t mask_words = 0;
		for (rdp_cp *cp : instances)
			if (r < cp->deferred.size())
			{
				views.push_back(cp->deferred[r].view());
				const rdpx::PassView &pv = views.back();
				prims += pv.num_prims;
				uploads += pv.num_uploads;
				for (uint32_t t = 0; t < pv.num_targets; t++)
				{
					const uint32_t tt = pv.target[t].tiles_x * pv.target[t].tiles_y;
					tiles += tt;
					mask_words += size_t(tt) * RDP_MASK_WORDS(pv.target_prims[t]);
				}
			}
		need.passes = std::max(need.passes, uint32_t(views.size()));
		need.prims = std::max(need.prims, prims);
		need.uploads = std::max(need.uploads, uploads);
		need.mask_words = std::max(need.mask_words, mask_words);
		need.tile_items = std::max(need.tile_items, tiles);
		need.staging = std::max(need.staging, rdpx::Executor::staging_bytes_for(views.data(), uint32_t(views.size())));
	}
	need.pairs = std::max(need.pairs, exec.initial_pairs);
	need.span_rows = std::max(need.span_rows, exec.initial_span_rows);
	return exec.ensure(need);
}

// ============================================================================ C ABI
extern "C" {

int rdp_device_is_supported(int device)
{
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
	return device >= 0 && device < n ? 1 : 0;
}

int rdp_cp_create(const rdp_create_info *info, rdp_cp **out)
{
	if (!info || !out) return RDP_ERR_INVALID;
	*out = nullptr;
	size_t rs = info->rdram_size, hs = info->hidden_rdram_size;
	const uint32_t known = RDP_CREATE_COMMAND_THREAD | RDP_CREATE_UPSCALING_2X | RDP_CREATE_UPSCALING_4X |
	                       RDP_CREATE_UPSCALING_8X | RDP_CREATE_SUPER_SAMPLED_READ_BACK | RDP_CREATE_SUPER_SAMPLED_DITHER;
	const bool upscaling = (info->flags & (RDP_CREATE_UPSCALING_2X | RDP_CREATE_UPSCALING_4X | RDP_CREATE_UPSCALING_8X)) != 0;
	if (!rs || (rs & (rs - 1)) || !hs || (hs & (hs - 1)) || rs > (64u << 20) || (info->flags & ~known) ||
	    (upscaling && hs != rs / 2) || (!upscaling && (info->flags & RDP_CREATE_SUPER_SAMPLED_READ_BACK)))
		return RDP_ERR_INVALID;
	if (!rdp_device_is_supported(info->device)) return RDP_ERR_UNSUPPORTED;
	rdp_cp *cp = new (std::nothrow) rdp_cp();
	if (!cp) return RDP_ERR_OOM;
	int r = cp->init(info);
	if (r == RDP_OK && (info->flags & RDP_CREATE_COMMAND_THREAD)) r = cp->start_command_thread();
	if (r != RDP_OK)
	{
		cp->destroy();
		delete cp;
		return r;
	}
	*out = cp;
	return RDP_OK;
}

void rdp_cp_destroy(rdp_cp *cp)
{
	if (!cp) return;
	cudaSetDevice(cp->device);
	cp->stop_command_thread();
	if (cp->batch)
	{
		// Finish the instance's deferred work (the batch's other instances keep theirs).
		cp->idle();
		auto &v = cp->batch->instances;
		v.erase(std::remove(v.begin(), v.end(), cp), v.end());
	}
	cp->destroy();
	delete cp;
}

int rdp_cp_enqueue(rdp_cp *cp, uint32_t num_words, const uint32_t *words)
{
	if (!cp || (num_words && !words)) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	return cp->api_enqueue(num_words, words);
}

int rdp_cp_signal_timeline(rdp_cp *cp, uint64_t *value)
{
	if (!cp) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	return cp->api_signal(value);
}

int rdp_cp_wait_timeline(rdp_cp *cp, uint64_t value, uint64_t timeout_ns)
{
	if (!cp) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	return cp->wait_timeline(value, timeout_ns);
}

int rdp_cp_flush(rdp_cp *cp)
{
	if (!cp) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	return cp->api_flush();
}

int rdp_cp_idle(rdp_cp *cp)
{
	if (!cp) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	return cp->idle();
}

int rdp_cp_begin_frame_context(rdp_cp *cp)
{
	if (!cp) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	return cp->api_flush();
}

int rdp_cp_set_quirks(rdp_cp *cp, uint32_t quirks)
{
	if (!cp) return RDP_ERR_INVALID;
	const uint32_t w[2] = { 0x04u << 24, quirks };
	cudaSetDevice(cp->device);
	return cp->api_enqueue(2, w);
}

int rdp_cp_set_validation_callback(rdp_cp *cp, rdp_validation_cb cb, void *user)
{
	if (!cp) return RDP_ERR_INVALID;
	cp->validation_cb = cb;
	cp->validation_user = user;
	return RDP_OK;
}

void *rdp_cp_begin_read_rdram(rdp_cp *cp)
{
	if (!cp) return nullptr;
	cudaSetDevice(cp->device);
	cp->sync_ring();
	if (cp->idle() != RDP_OK) return nullptr;
	return cp->host_rdram;
}

int rdp_cp_end_write_rdram(rdp_cp *cp)
{
	if (!cp) return RDP_ERR_INVALID;
	cp->sync_ring();
	cudaSetDevice(cp->device);
	if (cp->coherent)
	{
		// Pages are refreshed from the caller's RDRAM whenever the GPU reads them; this makes the
		// next pass refresh all of them (masked), for consumers that rely on the call.
		cp->refresh_all = true;
		return RDP_OK;
	}
	// Without mapped host memory: the whole RDRAM is uploaded in stream order, after the work
	// queued so far (a batch instance's deferred passes are launched first).
	int r = cp->sync_point();
	if (r != RDP_OK) return r;
	cp->host_rdram_dirty = true;
	return cp->flush();
}

void *rdp_cp_begin_read_hidden_rdram(rdp_cp *cp)
{
	if (!cp) return nullptr;
	cudaSetDevice(cp->device);
	cp->sync_ring();
	if (cp->idle() != RDP_OK) return nullptr;
	if (cudaMemcpy(cp->hidden_mirror.data(), cp->d_hidden, cp->hidden_size, cudaMemcpyDeviceToHost) != cudaSuccess)
		return nullptr;
	return cp->hidden_mirror.data();
}

int rdp_cp_end_write_hidden_rdram(rdp_cp *cp)
{
	if (!cp) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	cp->sync_ring();
	if (cp->idle() != RDP_OK) return cp->sticky_error;
	return cp->check(cudaMemcpy(cp->d_hidden, cp->hidden_mirror.data(), cp->hidden_size, cudaMemcpyHostToDevice));
}

size_t rdp_cp_get_rdram_size(rdp_cp *cp) { return cp ? cp->rdram_size : 0; }
size_t rdp_cp_get_hidden_rdram_size(rdp_cp *cp) { return cp ? cp->hidden_size : 0; }

int rdp_cp_get_tmem(rdp_cp *cp, uint16_t *out)
{
	if (!cp || !out) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	cp->sync_ring();
	int r = cp->idle();
	if (r != RDP_OK) return r;
	return cp->check(cudaMemcpy(out, cp->d_tmem, 4096, cudaMemcpyDeviceToHost));
}

uint32_t rdp_cp_get_scaling_factor(rdp_cp *cp) { return cp ? 1u << cp->up_log2 : 1u; }

static int read_upscaled(rdp_cp *cp, const uint8_t *src, uint64_t total, void *dst, uint64_t offset, uint64_t size)
{
	if (!cp || !dst || !cp->up_log2 || offset > total || size > total - offset) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	cp->sync_ring();
	int r = cp->idle();
	if (r != RDP_OK) return r;
	return cp->check(cudaMemcpy(dst, src + offset, size_t(size), cudaMemcpyDeviceToHost));
}
int rdp_cp_read_upscaled_rdram(rdp_cp *cp, void *dst, uint64_t offset, uint64_t size)
{
	return read_upscaled(cp, cp ? cp->d_ms_rdram : nullptr, cp ? uint64_t(cp->rdram_size) << (2 * cp->up_log2) : 0,
	                     dst, offset, size);
}
int rdp_cp_read_upscaled_hidden_rdram(rdp_cp *cp, void *dst, uint64_t offset, uint64_t size)
{
	return read_upscaled(cp, cp ? cp->d_ms_hidden : nullptr, cp ? uint64_t(cp->hidden_size) << (2 * cp->up_log2) : 0,
	                     dst, offset, size);
}

int rdp_cp_set_vi_register(rdp_cp *cp, uint32_t reg, uint32_t value)
{
	if (!cp || reg >= 14) return RDP_ERR_INVALID;
	cp->vi_regs[reg] = value;
	return RDP_OK;
}

void rdp_scanout_options_default(rdp_scanout_options *o)
{
	if (!o) return;
	memset(o, 0, sizeof(*o));
	o->upscale_deinterlacing = 1;
	o->vi_aa = o->vi_scale = o->vi_serrate = o->vi_dither_filter = o->vi_divot_filter = o->vi_gamma_dither = 1;
}

int rdp_cp_scanout_sync(rdp_cp *cp, const rdp_scanout_options *opts, uint32_t *rgba_out, uint32_t *width,
                        uint32_t *height)
{
	if (!cp || !rgba_out || !width || !height) return RDP_ERR_INVALID;
	rdp_scanout_options defaults;
	rdp_scanout_options_default(&defaults);
	cudaSetDevice(cp->device);
	cp->sync_ring(); // scanout drains the command ring first (rdp_device.cpp:1085)
	return cp->scanout(opts ? opts : &defaults, rgba_out, width, height);
}

int rdp_cp_scanout(rdp_cp *cp, const rdp_scanout_options *opts, rdp_vi_image *out)
{
	if (!cp || !out) return RDP_ERR_INVALID;
	rdp_scanout_options defaults;
	rdp_scanout_options_default(&defaults);
	cudaSetDevice(cp->device);
	cp->sync_ring();
	*out = rdp_vi_image{};
	const uint32_t *img = nullptr;
	uint32_t w = 0, h = 0;
	int r = cp->scanout_device(opts ? opts : &defaults, &img, &w, &h);
	if (r == RDP_OK) r = cp->check(cudaStreamSynchronize(cp->stream));
	if (r == RDP_OK && img) *out = rdp_vi_image{ img, w, h };
	return r;
}

int rdp_cp_scanout_async_buffer(rdp_cp *cp, const rdp_scanout_options *opts, rdp_vi_scanout_buffer *buf)
{
	if (!cp || !buf) return RDP_ERR_INVALID;
	rdp_scanout_options defaults;
	rdp_scanout_options_default(&defaults);
	cudaSetDevice(cp->device);
	cp->sync_ring();
	// A previous copy into the buffer must have finished before it is reused or grown.
	if (buf->fence && cp->check(cudaEventSynchronize(static_cast<cudaEvent_t>(buf->fence)))) return cp->sticky_error;
	const uint32_t *img = nullptr;
	uint32_t w = 0, h = 0;
	int r = cp->scanout_device(opts ? opts : &defaults, &img, &w, &h);
	buf->width = buf->height = 0;
	if (r != RDP_OK || !img) return r;
	const size_t n = size_t(w) * h;
	if (buf->capacity_pixels < n)
	{
		if (buf->pixels) cudaFreeHost(buf->pixels);
		buf->pixels = nullptr;
		buf->capacity_pixels = 0;
		if (cp->check(cudaMallocHost(&buf->pixels, n * 4))) return RDP_ERR_OOM;
		buf->capacity_pixels = n;
	}
	if (!buf->fence)
	{
		cudaEvent_t e = nullptr;
		if (cp->check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return cp->sticky_error;
		buf->fence = e;
	}
	if (cp->check(cudaMemcpyAsync(buf->pixels, img, n * 4, cudaMemcpyDeviceToHost, cp->stream)) ||
	    cp->check(cudaEventRecord(static_cast<cudaEvent_t>(buf->fence), cp->stream)))
		return cp->sticky_error;
	buf->width = w;
	buf->height = h;
	return RDP_OK;
}

int rdp_vi_scanout_buffer_wait(rdp_vi_scanout_buffer *buf, uint64_t timeout_ns)
{
	if (!buf) return RDP_ERR_INVALID;
	if (!buf->fence) return RDP_OK;
	const bool bounded = timeout_ns < (uint64_t(1) << 50);
	const auto deadline = std::chrono::steady_clock::now() + std::chrono::nanoseconds(bounded ? int64_t(timeout_ns) : 0);
	for (;;)
	{
		cudaError_t q = cudaEventQuery(static_cast<cudaEvent_t>(buf->fence));
		if (q == cudaSuccess) return RDP_OK;
		if (q != cudaErrorNotReady) return RDP_ERR_DEVICE;
		if (bounded && std::chrono::steady_clock::now() >= deadline) return RDP_ERR_TIMEOUT;
		std::this_thread::yield();
	}
}

void rdp_vi_scanout_buffer_release(rdp_vi_scanout_buffer *buf)
{
	if (!buf) return;
	if (buf->fence)
	{
		cudaEventSynchronize(static_cast<cudaEvent_t>(buf->fence));
		cudaEventDestroy(static_cast<cudaEvent_t>(buf->fence));
	}
	if (buf->pixels) cudaFreeHost(buf->pixels);
	*buf = rdp_vi_scanout_buffer{};
}

int rdp_cp_begin_vi_register_per_scanline(rdp_cp *cp, uint32_t flags)
{
	if (!cp) return RDP_ERR_INVALID;
	cp->vi_begin_per_scanline(flags);
	return RDP_OK;
}

int rdp_cp_set_vi_register_for_scanline(rdp_cp *cp, uint32_t reg_bit, uint32_t value)
{
	if (!cp) return RDP_ERR_INVALID;
	cp->vi_set_for_scanline(reg_bit, value);
	return RDP_OK;
}

int rdp_cp_latch_vi_register_for_scanline(rdp_cp *cp, uint32_t vi_line)
{
	if (!cp) return RDP_ERR_INVALID;
	cp->vi_latch_scanline(vi_line);
	return RDP_OK;
}

int rdp_cp_end_vi_register_per_scanline(rdp_cp *cp)
{
	if (!cp) return RDP_ERR_INVALID;
	cp->vi_end_per_scanline();
	return RDP_OK;
}

int rdp_cp_get_stats(rdp_cp *cp, rdp_stats *out)
{
	if (!cp || !out) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	cp->sync_ring();
	*out = cp->stats;
	unsigned long long counters[3] = { 0, 0, 0 };
	if (cudaMemcpy(counters, cp->d_fragments, sizeof(counters), cudaMemcpyDeviceToHost) != cudaSuccess) return RDP_ERR_DEVICE;
	out->fragments = counters[0];
	out->touched_tiles = counters[1];
	out->tile_instances = counters[2];
	out->reference_passes = cp->stats.reference_passes + ((cp->ref.prims || cp->ref.uploads) ? 1 : 0);
	if (!cp->batch) out->staging_bytes = cp->exec->staging_bytes;
	return RDP_OK;
}

// A CUDA graph of recorded launches.  It replays on the executor's stream with the
// executor's scratch buffers, so it is valid while the executor keeps its generation.
struct rdp_graph
{
	rdpx::Executor *exec = nullptr;
	// The processors whose passes the graph replays and the RDRAM ranges those passes write
	// (marked for copy-back after every replay).  A batch's graph looks its instances up in the
	// batch at replay, so an instance destroyed since the capture is skipped.
	rdp_batch *batch = nullptr;
	std::vector<std::pair<rdp_cp *, std::vector<std::pair<uint32_t, uint32_t>>>> written;
	uint64_t generation = 0;
	rdp_stats *stats = nullptr; // receives kernel_launches, when the graph belongs to one processor
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t gexec = nullptr;
	std::vector<void *> buffers;
	std::vector<std::pair<cudaEvent_t, cudaEvent_t>> shade_events, blend_events;
	uint32_t kernels = 0, shade_launches = 0;
	float last_shade_ms = 0.0f, last_blend_ms = 0.0f;
	cudaEvent_t ev[2] = { nullptr, nullptr };
};

static int build_graph(rdpx::Executor *exec, rdpx::CaptureSink &sink, rdp_stats *stats, rdp_graph **out)
{
	rdp_graph *g = new (std::nothrow) rdp_graph();
	if (!g) return RDP_ERR_OOM;
	g->exec = exec;
	g->generation = exec->generation;
	g->stats = stats;
	g->buffers.swap(sink.buffers);
	bool ok = cudaStreamBeginCapture(exec->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
	if (ok)
	{
		for (auto &L : sink.launches)
		{
			rdp_kernels_launch(&L, exec->stream);
			g->kernels += rdp_kernels_count(&L);
			if (L.num_prims && L.num_tile_items)
			{
				g->shade_events.emplace_back(L.shade_events[0], L.shade_events[1]);
				g->blend_events.emplace_back(L.blend_events[0], L.blend_events[1]);
				g->shade_launches++;
			}
			else
			{
				for (cudaEvent_t e : { L.shade_events[0], L.shade_events[1], L.blend_events[0], L.blend_events[1] })
					cudaEventDestroy(e);
			}
		}
		ok = cudaStreamEndCapture(exec->stream, &g->graph) == cudaSuccess;
	}
	sink.launches.clear();
	ok = ok && cudaGraphInstantiate(&g->gexec, g->graph, 0) == cudaSuccess;
	ok = ok && cudaEventCreate(&g->ev[0]) == cudaSuccess && cudaEventCreate(&g->ev[1]) == cudaSuccess;
	if (!ok)
	{
		cudaGetLastError();
		rdp_graph_destroy(g);
		return RDP_ERR_DEVICE;
	}
	*out = g;
	return RDP_OK;
}

int rdp_cp_capture_begin(rdp_cp *cp)
{
	if (!cp || cp->capturing || cp->batch || cp->ring || cp->up_log2) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	int r = cp->hard_flush();
	if (r != RDP_OK) return r;
	cp->capturing = true;
	cp->capture_sink = rdpx::CaptureSink{};
	return RDP_OK;
}

int rdp_cp_capture_end(rdp_cp *cp, rdp_graph **out)
{
	if (!cp || !out || !cp->capturing) return RDP_ERR_INVALID;
	cudaSetDevice(cp->device);
	int r = cp->hard_flush();
	cp->capturing = false;
	if (r != RDP_OK) return r;
	r = build_graph(cp->exec, cp->capture_sink, &cp->stats, out);
	if (r != RDP_OK) cp->sticky_error = r;
	else
	{
		(*out)->written.emplace_back(cp, std::move(cp->capture_written));
		cp->capture_written.clear();
	}
	return r;
}

int rdp_graph_replay(rdp_graph *g, uint32_t count, float *elapsed_ms)
{
	if (!g) return RDP_ERR_INVALID;
	rdpx::Executor *ex = g->exec;
	if (ex->generation != g->generation) return RDP_ERR_INVALID; // scratch was reallocated since capture
	cudaSetDevice(ex->device);
	if (cudaEventRecord(g->ev[0], ex->stream) != cudaSuccess) return RDP_ERR_DEVICE;
	for (uint32_t i = 0; i < count; i++)
		if (cudaGraphLaunch(g->gexec, ex->stream) != cudaSuccess) return RDP_ERR_DEVICE;
	if (cudaEventRecord(g->ev[1], ex->stream) != cudaSuccess) return RDP_ERR_DEVICE;
	if (cudaEventSynchronize(g->ev[1]) != cudaSuccess) return RDP_ERR_DEVICE;
	ex->kernel_launches += uint64_t(g->kernels) * count;
	if (g->stats) g->stats->kernel_launches += uint64_t(g->kernels) * count;
	// The replayed passes wrote their framebuffer ranges again: the next timeline value of each
	// processor copies them back to its RDRAM.
	for (auto &w : g->written)
	{
		if (g->batch && std::find(g->batch->instances.begin(), g->batch->instances.end(), w.first) ==
		                    g->batch->instances.end())
			continue;
		for (auto &rg : w.second)
		{
			if (w.first->coherent) w.first->mark_written_range(rg.first, rg.second);
			else w.first->merge_dirty(rg.first, rg.second);
		}
	}
	if (elapsed_ms && cudaEventElapsedTime(elapsed_ms, g->ev[0], g->ev[1]) != cudaSuccess) return RDP_ERR_DEVICE;
	// GPU time of the rasteriser launches of the last replay.
	g->last_shade_ms = 0.0f;
	g->last_blend_ms = 0.0f;
	for (auto &pr : g->shade_events)
	{
		float ms = 0.0f;
		if (cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) g->last_shade_ms += ms;
		else cudaGetLastError(); // keep the thread's last-error slot clean for other CUDA users
	}
	for (auto &pr : g->blend_events)
	{
		float ms = 0.0f;
		if (cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) g->last_blend_ms += ms;
		else cudaGetLastError();
	}
	return RDP_OK;
}

float rdp_graph_last_shade_ms(rdp_graph *g) { return g ? g->last_shade_ms : 0.0f; }
float rdp_graph_last_blend_ms(rdp_graph *g) { return g ? g->last_blend_ms : 0.0f; }
uint32_t rdp_graph_shade_launches(rdp_graph *g) { return g ? g->shade_launches : 0; }

uint32_t rdp_graph_kernel_count(rdp_graph *g) { return g ? g->kernels : 0; }

void rdp_graph_destroy(rdp_graph *g)
{
	if (!g) return;
	cudaSetDevice(g->exec->device);
	cudaStreamSynchronize(g->exec->stream);
	if (g->gexec) cudaGraphExecDestroy(g->gexec);
	if (g->graph) cudaGraphDestroy(g->graph);
	for (void *b : g->buffers) cudaFree(b);
	for (auto *list : { &g->shade_events, &g->blend_events })
		for (auto &pr : *list)
		{
			cudaEventDestroy(pr.first);
			cudaEventDestroy(pr.second);
		}
	for (auto e : g->ev)
		if (e) cudaEventDestroy(e);
	delete g;
}

int rdp_batch_create(const rdp_batch_create_info *info, rdp_batch **out)
{
	if (!info || !out) return RDP_ERR_INVALID;
	*out = nullptr;
	if (!rdp_device_is_supported(info->device)) return RDP_ERR_UNSUPPORTED;
	if (info->flags & ~uint32_t(RDP_BATCH_TILE_ORDER_LEARNED | RDP_BATCH_RECORD_TILE_CYCLES)) return RDP_ERR_INVALID;
	if (cudaSetDevice(info->device) != cudaSuccess) return RDP_ERR_UNSUPPORTED;
	rdp_batch *b = new (std::nothrow) rdp_batch();
	if (!b) return RDP_ERR_OOM;
	b->device = info->device;
	b->flags = info->flags;
	if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess || !b->exec.init(b->device, b->stream))
	{
		b->exec.destroy();
		if (b->stream) cudaStreamDestroy(b->stream);
		delete b;
		return RDP_ERR_DEVICE;
	}
	b->exec.cycles_requested = (info->flags & RDP_BATCH_RECORD_TILE_CYCLES) != 0;
	b->exec.record_cycles = b->exec.cycles_requested;
	if ((info->flags & RDP_BATCH_TILE_ORDER_LEARNED) && !b->exec.sched_enable(true, false, 1e-3f, 1))
	{
		b->exec.destroy();
		cudaStreamDestroy(b->stream);
		delete b;
		return RDP_ERR_DEVICE;
	}
	*out = b;
	return RDP_OK;
}

int rdp_batch_destroy(rdp_batch *b)
{
	if (!b) return RDP_ERR_INVALID;
	if (!b->instances.empty()) return RDP_ERR_INVALID;
	cudaSetDevice(b->device);
	b->exec.destroy();
	for (void *p : b->sink.buffers) cudaFree(p);
	cudaStreamDestroy(b->stream);
	delete b;
	return RDP_OK;
}

int rdp_batch_add_instance(rdp_batch *b, const rdp_create_info *info, rdp_cp **out)
{
	if (!b || !info || !out) return RDP_ERR_INVALID;
	*out = nullptr;
	size_t rs = info->rdram_size, hs = info->hidden_rdram_size;
	if (!rs || (rs & (rs - 1)) || !hs || (hs & (hs - 1)) || rs > (64u << 20) || info->flags != 0 ||
	    info->device != b->device)
		return RDP_ERR_INVALID;
	rdp_cp *cp = new (std::nothrow) rdp_cp();
	if (!cp) return RDP_ERR_OOM;
	int r = cp->init(info, b, &b->exec);
	if (r != RDP_OK)
	{
		cp->destroy();
		delete cp;
		return r;
	}
	b->instances.push_back(cp);
	*out = cp;
	return RDP_OK;
}

int rdp_batch_submit(rdp_batch *b)
{
	if (!b) return RDP_ERR_INVALID;
	cudaSetDevice(b->device);
	for (rdp_cp *cp : b->instances)
	{
		int r = cp->hard_flush();
		if (r != RDP_OK) return r;
	}
	return b->submit();
}

int rdp_batch_idle(rdp_batch *b)
{
	int r = rdp_batch_submit(b);
	if (r != RDP_OK) return r;
	if (cudaStreamSynchronize(b->stream) != cudaSuccess) return b->sticky_error = RDP_ERR_DEVICE;
	for (rdp_cp *cp : b->instances)
	{
		uint64_t v = 0;
		if ((r = cp->signal_timeline(&v)) != RDP_OK || (r = cp->wait_timeline(v, UINT64_MAX / 2)) != RDP_OK) return r;
	}
	if (!b->capturing && !b->exec.adapt_pairs()) return b->sticky_error = RDP_ERR_DEVICE;
	b->exec.tune_epoch();
	if (b->exec.take_device_error()) return b->sticky_error = RDP_ERR_TIMEOUT;
	return RDP_OK;
}

int rdp_batch_get_stats(rdp_batch *b, rdp_batch_stats *out)
{
	if (!b || !out) return RDP_ERR_INVALID;
	out->instances = b->instances.size();
	out->rounds = b->rounds;
	out->passes = b->passes;
	out->kernel_launches = b->exec.kernel_launches;
	out->staging_bytes = b->exec.staging_bytes;
	return RDP_OK;
}

int rdp_batch_capture_begin(rdp_batch *b)
{
	if (!b || b->capturing) return RDP_ERR_INVALID;
	int r = rdp_batch_submit(b);
	if (r != RDP_OK) return r;
	b->capturing = true;
	b->sink = rdpx::CaptureSink{};
	return RDP_OK;
}

int rdp_batch_capture_end(rdp_batch *b, rdp_graph **out)
{
	if (!b || !out || !b->capturing) return RDP_ERR_INVALID;
	int r = rdp_batch_submit(b);
	b->capturing = false;
	if (r != RDP_OK) return r;
	r = build_graph(&b->exec, b->sink, nullptr, out);
	for (rdp_cp *cp : b->instances)
	{
		if (r == RDP_OK && !cp->capture_written.empty()) (*out)->written.emplace_back(cp, std::move(cp->capture_written));
		cp->capture_written.clear();
	}
	if (r == RDP_OK) (*out)->batch = b;
	return r;
}

int rdp_set_shade_variant(int device, int variant)
{
	if (device < 0 || device >= 64 || variant < -1 || variant >= RDP_SHADE_VARIANTS) return RDP_ERR_INVALID;
	rdpx::shade_variant_choice(device) = variant;
	return RDP_OK;
}

int rdp_get_shade_variant(int device)
{
	if (device < 0 || device >= 64) return -1;
	return rdpx::shade_variant_choice(device);
}

int rdp_set_shade_order(int device, int order)
{
	if (device < 0 || device >= 64 || order < 0 || order > 2) return RDP_ERR_INVALID;
	rdpx::shade_order_choice(device) = order;
	return RDP_OK;
}

int rdp_get_shade_order(int device)
{
	if (device < 0 || device >= 64) return -1;
	return rdpx::shade_order_choice(device);
}

int rdp_batch_set_schedule(rdp_batch *b, int learned_order, int train, float learning_rate, uint32_t train_stride)
{
	if (!b || learning_rate < 0.0f) return RDP_ERR_INVALID;
	cudaSetDevice(b->device);
	if (!learned_order && !train && !b->exec.sched_ready) return RDP_OK;
	return b->exec.sched_enable(learned_order != 0, train != 0, learning_rate, train_stride) ? RDP_OK : RDP_ERR_DEVICE;
}

int rdp_batch_get_model(rdp_batch *b, float *params, float *last_loss)
{
	if (!b || !params) return RDP_ERR_INVALID;
	cudaSetDevice(b->device);
	if (!b->exec.sched_ready && !b->exec.sched_enable(false, false, 0.0f, 1)) return RDP_ERR_DEVICE;
	if (cudaStreamSynchronize(b->stream) != cudaSuccess) return RDP_ERR_DEVICE;
	if (cudaMemcpy(params, b->exec.sched.w32, sizeof(float) * RDP_MLP_PARAMS, cudaMemcpyDeviceToHost) != cudaSuccess)
		return RDP_ERR_DEVICE;
	if (last_loss)
	{
		float l[2] = { 0.0f, 0.0f };
		if (cudaMemcpy(l, b->exec.sched.loss, sizeof(l), cudaMemcpyDeviceToHost) != cudaSuccess) return RDP_ERR_DEVICE;
		*last_loss = l[1] > 0.0f ? l[0] / l[1] : 0.0f;
	}
	return RDP_OK;
}

int rdp_batch_set_model(rdp_batch *b, const float *params)
{
	if (!b || !params) return RDP_ERR_INVALID;
	cudaSetDevice(b->device);
	rdpx::Executor &ex = b->exec;
	if (!ex.sched_ready && !ex.sched_enable(false, false, 0.0f, 1)) return RDP_ERR_DEVICE;
	std::vector<__half> h(RDP_MLP_PARAMS);
	for (int i = 0; i < RDP_MLP_PARAMS; i++) h[i] = __float2half_rn(params[i]);
	if (cudaStreamSynchronize(b->stream) != cudaSuccess ||
	    cudaMemcpy(ex.sched.w32, params, sizeof(float) * RDP_MLP_PARAMS, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(ex.sched.w16, h.data(), sizeof(__half) * RDP_MLP_PARAMS, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemset(ex.sched.adam_m, 0, sizeof(float) * RDP_MLP_PARAMS) != cudaSuccess ||
	    cudaMemset(ex.sched.adam_v, 0, sizeof(float) * RDP_MLP_PARAMS) != cudaSuccess ||
	    cudaMemset(ex.sched.adam_t, 0, sizeof(uint32_t)) != cudaSuccess)
		return RDP_ERR_DEVICE;
	return RDP_OK;
}

// Runs the MLP kernels on caller data (weights rounded to FP16 as the scheduler stores them).
static int mlp_call(int device, const float *params, const float *features, const float *targets, uint32_t n,
                    float *grads, float *loss, float *out)
{
	if (!params || !features || !n || cudaSetDevice(device) != cudaSuccess) return RDP_ERR_INVALID;
	std::vector<__half> h(RDP_MLP_PARAMS);
	for (int i = 0; i < RDP_MLP_PARAMS; i++) h[i] = __float2half_rn(params[i]);
	__half *dw = nullptr;
	float *df = nullptr, *dt = nullptr, *dg = nullptr, *dl = nullptr, *dout = nullptr;
	int r = RDP_ERR_DEVICE;
	cudaStream_t s = nullptr;
	if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
	    cudaMalloc(&dw, sizeof(__half) * RDP_MLP_PARAMS) == cudaSuccess &&
	    cudaMalloc(&df, sizeof(float) * RDP_MLP_IN * size_t(n)) == cudaSuccess &&
	    cudaMemcpy(dw, h.data(), sizeof(__half) * RDP_MLP_PARAMS, cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemcpy(df, features, sizeof(float) * RDP_MLP_IN * size_t(n), cudaMemcpyHostToDevice) == cudaSuccess)
	{
		if (out)
		{
			if (cudaMalloc(&dout, sizeof(float) * n) == cudaSuccess &&
			    rdp_sched_launch_forward(dw, df, n, dout, s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess &&
			    cudaMemcpy(out, dout, sizeof(float) * n, cudaMemcpyDeviceToHost) == cudaSuccess)
				r = RDP_OK;
		}
		else if (targets && grads &&
		         cudaMalloc(&dt, sizeof(float) * n) == cudaSuccess &&
		         cudaMalloc(&dg, sizeof(float) * RDP_MLP_PARAMS) == cudaSuccess && cudaMalloc(&dl, 2 * sizeof(float)) == cudaSuccess &&
		         cudaMemcpy(dt, targets, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
		         cudaMemset(dg, 0, sizeof(float) * RDP_MLP_PARAMS) == cudaSuccess && cudaMemset(dl, 0, 2 * sizeof(float)) == cudaSuccess &&
		         rdp_sched_launch_grad(dw, df, dt, n, dg, dl, s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess &&
		         cudaMemcpy(grads, dg, sizeof(float) * RDP_MLP_PARAMS, cudaMemcpyDeviceToHost) == cudaSuccess)
		{
			float l[2];
			if (cudaMemcpy(l, dl, sizeof(l), cudaMemcpyDeviceToHost) == cudaSuccess)
			{
				if (loss) *loss = l[1] > 0.0f ? l[0] / l[1] : 0.0f;
				r = RDP_OK;
			}
		}
	}
	cudaGetLastError();
	cudaFree(dw);
	cudaFree(df);
	cudaFree(dt);
	cudaFree(dg);
	cudaFree(dl);
	cudaFree(dout);
	if (s) cudaStreamDestroy(s);
	return r;
}

int rdp_mlp_gradients(int device, const float *params, const float *features, const float *targets, uint32_t n,
                      float *grads, float *loss)
{
	if (!targets || !grads) return RDP_ERR_INVALID;
	return mlp_call(device, params, features, targets, n, grads, loss, nullptr);
}

int rdp_mlp_forward(int device, const float *params, const float *features, uint32_t n, float *out)
{
	if (!out) return RDP_ERR_INVALID;
	return mlp_call(device, params, features, nullptr, n, nullptr, nullptr, out);
}

int rdp_batch_get_tile_samples(rdp_batch *b, float *features, float *predicted, uint32_t *cycles, uint32_t max_tiles,
                               uint32_t *count)
{
	if (!b || !count) return RDP_ERR_INVALID;
	cudaSetDevice(b->device);
	rdpx::Executor &ex = b->exec;
	*count = 0;
	if (cudaStreamSynchronize(b->stream) != cudaSuccess) return RDP_ERR_DEVICE;
	uint32_t ctrl[5];
	if (cudaMemcpy(ctrl, ex.d_ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost) != cudaSuccess) return RDP_ERR_DEVICE;
	uint32_t n = std::min(ctrl[3], max_tiles);
	if (ctrl[1]) n = 0;
	if (!n) return RDP_OK;
	std::vector<uint32_t> items(n);
	if (cudaMemcpy(items.data(), ex.d_nonempty, 4 * size_t(n), cudaMemcpyDeviceToHost) != cudaSuccess) return RDP_ERR_DEVICE;
	if (features || predicted)
	{
		if (!ex.sched_ready || !ex.sched.features) return RDP_ERR_INVALID;
		if (features)
		{
			std::vector<float> all(size_t(ex.sched_capacity) * RDP_MLP_IN);
			if (cudaMemcpy(all.data(), ex.sched.features, sizeof(float) * all.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
				return RDP_ERR_DEVICE;
			for (uint32_t k = 0; k < n; k++)
				for (int f = 0; f < RDP_MLP_IN; f++)
					features[size_t(k) * RDP_MLP_IN + f] = items[k] < ex.sched_capacity ? all[size_t(items[k]) * RDP_MLP_IN + f] : 0.0f;
		}
		if (predicted && cudaMemcpy(predicted, ex.sched.pred, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
			return RDP_ERR_DEVICE;
	}
	if (cycles)
	{
		if (!ex.record_cycles) return RDP_ERR_INVALID;
		std::vector<uint32_t> all(ex.caps.tile_items);
		if (cudaMemcpy(all.data(), ex.d_tile_cycles, 4 * all.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
			return RDP_ERR_DEVICE;
		for (uint32_t k = 0; k < n; k++) cycles[k] = items[k] < all.size() ? all[items[k]] : 0u;
	}
	*count = n;
	return RDP_OK;
}

int rdp_serve_run(rdp_batch *b, rdp_cp *const *instances, uint32_t num_instances, const rdp_serve_request *requests,
                  uint32_t num_requests, const rdp_serve_config *config, rdp_serve_result *results,
                  rdp_serve_stats *stats)
{
	if (!b || !instances || !num_instances || (num_requests && (!requests || !results)) || !config) return RDP_ERR_INVALID;
	for (uint32_t i = 0; i < num_instances; i++)
		if (!instances[i] || instances[i]->batch != b) return RDP_ERR_INVALID;
	for (uint32_t r = 0; r < num_requests; r++)
	{
		if (requests[r].instance >= num_instances || (requests[r].num_words && !requests[r].words)) return RDP_ERR_INVALID;
		if (r && requests[r].arrival_s < requests[r - 1].arrival_s) return RDP_ERR_INVALID; // sorted by arrival
	}
	cudaSetDevice(b->device);
	using clock = std::chrono::steady_clock;
	const auto t0 = clock::now();
	auto now_s = [&] { return std::chrono::duration<double>(clock::now() - t0).count(); };
	// Footprint estimate: primitive records, staging, ~8 shaded (primitive, tile) pairs and ~24
	// span rows per primitive.
	auto footprint = [](const rdp_serve_request &q) -> uint64_t {
		if (q.footprint_bytes) return q.footprint_bytes;
		uint64_t prims = q.num_words / 20 + 1;
		return prims * (336 + 8 * 520 + 24 * RDP_SPAN_ROW_BYTES) + uint64_t(q.num_words) * 4;
	};
	struct Flight
	{
		uint32_t req;
		uint64_t value, bytes;
	};
	std::deque<uint32_t> waiting;
	std::vector<Flight> flying;
	std::vector<uint32_t> admit, group_of(num_instances, UINT32_MAX);
	std::vector<std::vector<uint32_t>> groups;
	std::vector<uint64_t> admitted_value(num_requests, 0);
	std::vector<int> admitted_status(num_requests, RDP_OK);
	uint32_t next = 0, done = 0;
	uint64_t in_bytes = 0;
	rdp_serve_stats st = {};
	int r = RDP_OK;
	while (done < num_requests)
	{
		const double t = now_s();
		if (t > config->timeout_s)
		{
			r = RDP_ERR_TIMEOUT;
			break;
		}
		bool progress = false;
		while (next < num_requests && requests[next].arrival_s <= t) waiting.push_back(next++);
		// Completions: event queries only (no submission happens here).
		for (size_t k = 0; k < flying.size();)
		{
			rdp_cp *cp = instances[requests[flying[k].req].instance];
			int w = cp->poll_timeline(flying[k].value);
			if (w == RDP_ERR_TIMEOUT)
			{
				k++;
				continue;
			}
			if (w != RDP_OK)
			{
				r = w;
				break;
			}
			rdp_serve_result &res = results[flying[k].req];
			res.done_s = now_s();
			res.latency_s = res.done_s - requests[flying[k].req].arrival_s;
			in_bytes -= flying[k].bytes;
			flying[k] = flying.back();
			flying.pop_back();
			done++;
			progress = true;
		}
		if (r != RDP_OK) break;
		// Admission in arrival order while the budget has room (at least one frame always fits).
		// The admitted requests are chosen first; their command words are then parsed on the
		// batch's parse threads, one task per instance (its requests in arrival order), and all
		// tasks have finished before the loop submits or polls again.
		admit.clear();
		while (!waiting.empty())
		{
			const uint32_t q = waiting.front();
			const uint64_t fp = footprint(requests[q]);
			const size_t in_flight = flying.size() + admit.size();
			if (in_flight && (in_bytes + fp > config->hbm_budget_bytes ||
			                  (config->max_in_flight && in_flight >= config->max_in_flight)))
				break;
			admit.push_back(q);
			in_bytes += fp;
			waiting.pop_front();
		}
		if (!admit.empty())
		{
			groups.clear();
			for (uint32_t q : admit)
			{
				const uint32_t inst = requests[q].instance;
				if (group_of[inst] == UINT32_MAX)
				{
					group_of[inst] = uint32_t(groups.size());
					groups.emplace_back();
				}
				groups[group_of[inst]].push_back(q);
			}
			b->parse_pool.run(uint32_t(groups.size()), [&](uint32_t g) {
				cudaSetDevice(b->device);
				for (uint32_t q : groups[g])
				{
					rdp_cp *cp = instances[requests[q].instance];
					int e = cp->enqueue(requests[q].num_words, requests[q].words);
					if (e == RDP_OK) e = cp->signal_timeline(&admitted_value[q]);
					admitted_status[q] = e;
				}
			});
			const double t_admit = now_s();
			for (const auto &grp : groups) group_of[requests[grp.front()].instance] = UINT32_MAX;
			for (uint32_t q : admit)
			{
				if (admitted_status[q] != RDP_OK && r == RDP_OK) r = admitted_status[q];
				results[q].admit_s = t_admit;
				flying.push_back(Flight{ q, admitted_value[q], footprint(requests[q]) });
			}
			st.max_in_flight = std::max<uint64_t>(st.max_in_flight, flying.size());
			st.max_footprint = std::max(st.max_footprint, in_bytes);
		}
		if (r != RDP_OK) break;
		if (!admit.empty())
		{
			// One submission for everything admitted in this pass: the new frames share launches.
			if ((r = b->submit()) != RDP_OK) break;
			st.submits++;
			progress = true;
		}
		if (!progress) std::this_thread::yield();
	}
	st.elapsed_s = now_s();
	if (stats) *stats = st;
	return r;
}

int rdp_batch_enqueue_many(rdp_batch *b, uint32_t count, rdp_cp *const *instances, const uint32_t *const *words,
                           const uint32_t *num_words, uint64_t *timeline_values, uint32_t threads)
{
	if (!b || (count && (!instances || !words || !num_words))) return RDP_ERR_INVALID;
	// Each instance is parsed by exactly one thread: a handle given twice would put two threads
	// on one recorder.  Checked before any handle is dereferenced or any thread starts.
	{
		std::vector<rdp_cp *> sorted(instances, instances + count);
		std::sort(sorted.begin(), sorted.end());
		if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) return RDP_ERR_INVALID;
	}
	for (uint32_t i = 0; i < count; i++)
		if (!instances[i] || instances[i]->batch != b) return RDP_ERR_INVALID;
	cudaSetDevice(b->device);
	std::vector<int> status(count, RDP_OK);
	auto one = [&](uint32_t i) {
		cudaSetDevice(b->device);
		rdp_cp *cp = instances[i];
		int r = cp->enqueue(num_words[i], words[i]);
		uint64_t v = 0;
		if (r == RDP_OK && timeline_values) r = cp->signal_timeline(&v);
		if (timeline_values) timeline_values[i] = v;
		status[i] = r;
	};
	if (!threads)
		b->parse_pool.run(count, one); // the batch's persistent parse threads (one per core, at most 16)
	else
	{
		threads = std::min(threads, std::max(count, 1u));
		std::atomic<uint32_t> next(0);
		auto work = [&] {
			for (uint32_t i; (i = next.fetch_add(1)) < count;) one(i);
		};
		std::vector<std::thread> pool;
		for (uint32_t t = 1; t < threads; t++) pool.emplace_back(work);
		work();
		for (auto &t : pool) t.join();
	}
	for (int r : status)
		if (r != RDP_OK) return r;
	return RDP_OK;
}

} // extern "C"
