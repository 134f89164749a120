/*
 * Launch executor of the GB300 RDP path: packs one or more recorded passes --
 * each from a different emulator instance -- into one staging buffer, copies it
 * to the device with one H2D copy and launches the kernel chain once for all of
 * them (rdp_kernels.cu).  A stand-alone command processor owns an executor and
 * submits one pass per launch; a batch shares one executor between its
 * instances and submits one pass of every instance per launch.
 *
 * Device buffers grow on demand.  Growth changes the executor's generation;
 * CUDA graphs recorded against an older generation refuse to replay.
 */
#ifndef RDP_EXEC_H
#define RDP_EXEC_H

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "rdp_types.h"
#include "rdp_kernels.h"
#include "sched.h"

namespace rdpx {

static inline size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

constexpr uint32_t kMaxTargets = 8;

// Persistent host worker threads for data-parallel host work (filling a launch's staging
// buffer): run(n, fn) calls fn(0..n-1) spread over the workers and the calling thread and
// returns when all calls have finished.  Workers start on first use.
class HostPool
{
public:
	~HostPool()
	{
		{
			std::lock_guard<std::mutex> lk(mu_);
			stop_ = true;
		}
		cv_.notify_all();
		for (auto &t : workers_) t.join();
	}

	void run(uint32_t n, const std::function<void(uint32_t)> &fn)
	{
		if (n <= 1 || max_workers() == 0)
		{
			for (uint32_t i = 0; i < n; i++) fn(i);
			return;
		}
		start();
		{
			std::lock_guard<std::mutex> lk(mu_);
			fn_ = &fn;
			n_ = n;
			next_.store(0);
			busy_ = uint32_t(workers_.size());
			gen_++;
		}
		cv_.notify_all();
		drain();
		std::unique_lock<std::mutex> lk(mu_);
		done_cv_.wait(lk, [&] { return busy_ == 0; });
		fn_ = nullptr;
	}

private:
	static uint32_t max_workers()
	{
		const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
		return std::min(hw, 16u) - 1;
	}
	void start()
	{
		if (!workers_.empty()) return;
		for (uint32_t t = 0; t < max_workers(); t++) workers_.emplace_back([this] { loop(); });
	}
	void drain()
	{
		for (;;)
		{
			const uint32_t i = next_.fetch_add(1);
			if (i >= n_) break;
			(*fn_)(i);
		}
	}
	void loop()
	{
		uint64_t seen = 0;
		for (;;)
		{
			{
				std::unique_lock<std::mutex> lk(mu_);
				cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
				if (stop_) return;
				seen = gen_;
			}
			drain();
			std::lock_guard<std::mutex> lk(mu_);
			if (--busy_ == 0) done_cv_.notify_all();
		}
	}

	std::vector<std::thread> workers_;
	std::mutex mu_;
	std::condition_variable cv_, done_cv_;
	const std::function<void(uint32_t)> *fn_ = nullptr;
	uint32_t n_ = 0, busy_ = 0;
	std::atomic<uint32_t> next_{ 0 };
	uint64_t gen_ = 0;
	bool stop_ = false;
};

// One recorded pass of an instance, as plain pointers into the recorder's buffers.
// A pass may draw into several colour images ("targets") whose memory does not
// overlap; each target becomes one RdpPass of the launch.  Its primitives are grouped
// by target: target t owns prims [sum(target_prims[<t]), +target_prims[t]).  The
// descriptors carry the instance's pointers; the executor fills in the bases.  The
// pass's TMEM uploads are applied by the first descriptor.
struct PassView
{
	RdpPass target[kMaxTargets];
	uint32_t target_prims[kMaxTargets];
	uint32_t num_targets;
	const RdpPrimIn *prims;
	uint32_t num_prims;
	const uint32_t *words;
	uint32_t num_words;
	const uint32_t *state_blocks;
	uint32_t num_state_blocks;
	const RdpTile *tilesets;
	uint32_t num_tilesets;
	const RdpUpload *uploads;
	uint32_t num_uploads;
	bool fill_only; // every primitive is drawn by the fill pipe (cycle type 3)
};

// An owned copy of a recorded pass (batched instances defer their passes).
struct PassPacket
{
	std::vector<RdpPass> targets;
	std::vector<uint32_t> target_prims;
	std::vector<RdpPrimIn> prims;
	std::vector<uint32_t> words, state_blocks;
	std::vector<RdpTile> tilesets;
	std::vector<RdpUpload> uploads;
	std::vector<uint32_t> read_pages; // RDRAM pages refreshed from the caller's memory before the pass
	bool fill_only = false;

	PassView view() const
	{
		PassView v;
		v.num_targets = uint32_t(targets.size());
		for (uint32_t t = 0; t < v.num_targets; t++)
		{
			v.target[t] = targets[t];
			v.target_prims[t] = target_prims[t];
		}
		v.prims = prims.data();
		v.num_prims = uint32_t(prims.size());
		v.words = words.data();
		v.num_words = uint32_t(words.size());
		v.state_blocks = state_blocks.data();
		v.num_state_blocks = uint32_t(state_blocks.size() / RDP_STATE_BLOCK_WORDS);
		v.tilesets = tilesets.data();
		v.num_tilesets = uint32_t(tilesets.size() / 8);
		v.uploads = uploads.data();
		v.num_uploads = uint32_t(uploads.size());
		v.fill_only = fill_only;
		return v;
	}
};

struct ExecCaps
{
	uint32_t passes = 0, descs = 0, prims = 0, tile_items = 0, pairs = 0, span_rows = 0, uploads = 0;
	size_t mask_words = 0; // tiles x each pass's bitmask words, summed over a launch
	size_t staging = 0;
};

// Span rows a launch buffer starts with (RDP_SPAN_ROW_BYTES each); batches grow it at idle to
// the largest count a launch needed.
constexpr uint32_t kInitialSpanRows = 1u << 21;

// Launches recorded for a CUDA graph, with their device-resident inputs.
struct CaptureSink
{
	std::vector<RdpLaunch> launches;
	std::vector<void *> buffers;
};

// Process-wide choice of the k_shade variant per device: -1 until tuned (or forced).
int &shade_variant_choice(int device);
int &shade_order_choice(int device);

// Autotuner of the shading kernel.  Tuning runs for RDP_SHADE_VARIANTS epochs (an epoch
// ends at each sync point: idle); in epoch e the i-th rasterising launch uses variant
// (i + e) mod RDP_SHADE_VARIANTS, so over the epochs every variant runs every launch
// position of a repeating frame once.  Each sampled launch's k_shade time (CUDA events on
// the stream) and pair count (written by k_scan) are summed per variant; the variant with
// the least time per pair is kept for the device.  The variants compute identical results,
// so tuning never changes output.
struct ShadeTuner
{
	static constexpr uint32_t kMaxSamplesPerEpoch = 64;
	bool active = false;
	int epoch = 0;
	uint32_t in_epoch = 0;
	uint64_t samples_taken = 0;
	struct Sample
	{
		int variant;
		cudaEvent_t ev[2];
		uint32_t slot;
	};
	std::vector<Sample> pending;
	std::vector<cudaEvent_t> pool;
	double ms[RDP_SHADE_VARIANTS] = {}, pairs[RDP_SHADE_VARIANTS] = {};
	int count[RDP_SHADE_VARIANTS] = {};

	cudaEvent_t event()
	{
		if (!pool.empty())
		{
			cudaEvent_t e = pool.back();
			pool.pop_back();
			return e;
		}
		cudaEvent_t e = nullptr;
		cudaEventCreate(&e);
		return e;
	}
	void destroy()
	{
		for (auto &sm : pending)
		{
			cudaEventDestroy(sm.ev[0]);
			cudaEventDestroy(sm.ev[1]);
		}
		for (auto e : pool) cudaEventDestroy(e);
		pending.clear();
		pool.clear();
	}
};

struct Executor
{
	int device = 0;
	cudaStream_t stream = nullptr;
	ExecCaps caps;
	uint64_t generation = 0;
	uint64_t kernel_launches = 0, staging_bytes = 0, launches = 0;
	uint32_t shade_ctas_v[RDP_SHADE_VARIANTS] = {}, blend_ctas = 0, blend_kernel = 0;
	bool failed = false;
	ShadeTuner tuner;
	HostPool pool;                                      // staging fill of large launches
	static constexpr size_t kParallelFillBytes = 1u << 20;
	uint32_t *d_pair_log = nullptr; // [256]
	// Launch log for profiling (RDP_LAUNCH_LOG=<file>): the pair count of every launch that runs
	// outside a capture and is not a tuning sample is appended to the file at the next sync point,
	// so that per-launch hardware counters can be scaled to per-pair figures.
	FILE *launch_log = nullptr;
	uint32_t *d_launch_pairs = nullptr; // [kLaunchLogSlots]
	static constexpr uint32_t kLaunchLogSlots = 4096;
	std::vector<std::pair<uint64_t, uint32_t>> launch_log_pending; // (launch number, slot)
	// Size thresholds of the shading orders (RDP_SHADE_PERM_MIN_PRIMS, RDP_SHADE_QUEUE_MIN
	// override them): primitive-major order for launches of at least perm_min_prims primitives,
	// per-SM queues for launches of at least queue_min pairs per k_shade CTA.
	uint32_t perm_min_prims = 16384, queue_min = 64;
	// Pair-scratch and span-row capacities a new executor starts with (RDP_PAIR_CAPACITY and
	// RDP_SPAN_ROW_CAPACITY override them; launches beyond them take the fused fallback).
	uint32_t initial_pairs = 1u << 20, initial_span_rows = kInitialSpanRows;
	bool fused_only = false; // RDP_RASTER_PATH=fused: the pair scratch never grows
	uint32_t *d_queues = nullptr, num_queues = 0; // per-SM work queues of k_shade + used-up bitmask
	size_t queue_bytes() const { return (size_t(num_queues) + (num_queues + 31) / 32) * 4; }

	RdpPrimGeom *d_geom = nullptr;
	RdpPrimAttr *d_attr = nullptr;
	RdpPrimShade *d_shade = nullptr;
	uint32_t *d_masks = nullptr, *d_tmem_keep = nullptr;
	uint32_t *d_tile_counts = nullptr, *d_pair_offsets = nullptr, *d_ctrl = nullptr;
	uint32_t *d_tile_order = nullptr, *d_tile_cycles = nullptr, *d_nonempty = nullptr, *d_scan_blocks = nullptr;
	uint32_t *d_prim_pairs = nullptr, *d_prim_offsets = nullptr, *d_prim_blocks = nullptr;
	uint32_t *d_prim_rows = nullptr; // first span row of each primitive
	void *d_spans = nullptr;         // span rows written by k_bin
	uint4 *d_shade_list = nullptr; // primitive-major shading records
	uint2 *d_pairs = nullptr;
	uint2 *d_scratch = nullptr; // shaded records, 64 per pair
	// Launch inputs are copied on copy_stream into a ring of kStagingSlots device slots, so that the
	// copies of the next launches overlap this launch's kernels (a sync point's large round follows
	// small ones: its copy starts while the previous sync point still renders).  slot_copied[s]
	// orders the kernels after the copy; slot_free[s] (recorded after the kernels that read slot s)
	// orders the next copy into it.
	static constexpr int kStagingSlots = 4;
	uint8_t *d_staging = nullptr; // kStagingSlots slots of caps.staging bytes
	cudaStream_t copy_stream = nullptr;
	// The TMEM kernels of a rasterising launch run on side_stream, overlapping set-up, binning,
	// span rows, scans and pair expansion (none of which reads TMEM); shading waits for them.
	cudaStream_t side_stream = nullptr;
	cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
	cudaEvent_t slot_copied[kStagingSlots] = {}, slot_free[kStagingSlots] = {};
	int staging_slot = 0;

	// Pinned host staging buffers, used round-robin; a buffer is reused once the H2D copy
	// that read it has completed.  Up to kMaxStaging of them let the host record launches
	// ahead of the GPU (the serving loop keeps admitting while earlier launches run).
	static constexpr size_t kMaxStaging = 8;
	struct Staging
	{
		uint8_t *h = nullptr;
		size_t size = 0;
		cudaEvent_t done = nullptr;
		bool in_flight = false;
	};
	std::vector<Staging> staging;
	size_t staging_next = 0, staging_largest = 0;

	// A host staging buffer of at least `bytes` whose previous copy has completed.
	Staging *take_staging(size_t bytes)
	{
		Staging *pick = nullptr;
		for (size_t k = 0; k < staging.size() && !pick; k++)
		{
			Staging &st = staging[(staging_next + k) % staging.size()];
			if (!st.in_flight || cudaEventQuery(st.done) == cudaSuccess)
			{
				st.in_flight = false;
				pick = &st;
			}
		}
		cudaGetLastError();
		if (!pick && staging.size() < kMaxStaging)
		{
			staging.emplace_back();
			pick = &staging.back();
			if (check(cudaEventCreateWithFlags(&pick->done, cudaEventDisableTiming))) return nullptr;
		}
		if (!pick)
		{
			pick = &staging[staging_next % staging.size()];
			if (check(cudaEventSynchronize(pick->done))) return nullptr;
			pick->in_flight = false;
		}
		staging_next = size_t(pick - staging.data()) + 1;
		if (pick->size < bytes)
		{
			// A new or grown buffer takes the largest size any buffer has needed, so that
			// the ring stops reallocating (cudaFreeHost waits for the device) once warm.
			size_t n = std::max(bytes, std::max(staging_largest, pick->size + pick->size / 2));
			if (pick->h) cudaFreeHost(pick->h);
			pick->h = nullptr;
			pick->size = 0;
			if (check(cudaMallocHost(&pick->h, n))) return nullptr;
			pick->size = n;
			staging_largest = std::max(staging_largest, n);
		}
		return pick;
	}

	bool record_cycles = false, cycles_requested = false;

	// Learned tile order (sched.h): model and per-tile buffers, allocated on first use.
	bool sched_ready = false;
	RdpSchedDev sched = {};
	uint32_t sched_capacity = 0;

	bool sched_enable(bool order, bool train, float lr, uint32_t stride)
	{
		if (!sched_ready)
		{
			if (check(cudaMalloc(&sched.w16, sizeof(__half) * RDP_MLP_PARAMS)) ||
			    check(cudaMalloc(&sched.w32, sizeof(float) * RDP_MLP_PARAMS)) ||
			    check(cudaMalloc(&sched.adam_m, sizeof(float) * RDP_MLP_PARAMS)) ||
			    check(cudaMalloc(&sched.adam_v, sizeof(float) * RDP_MLP_PARAMS)) ||
			    check(cudaMalloc(&sched.grad, sizeof(float) * RDP_MLP_PARAMS)) ||
			    check(cudaMalloc(&sched.adam_t, sizeof(uint32_t))) || check(cudaMalloc(&sched.loss, 2 * sizeof(float))) ||
			    check(cudaMalloc(&sched.hist, sizeof(uint32_t) * RDP_SCHED_BUCKETS)) ||
			    check(cudaMalloc(&sched.cursor, sizeof(uint32_t) * RDP_SCHED_BUCKETS)))
				return false;
			if (check(cudaMemsetAsync(sched.loss, 0, 2 * sizeof(float), stream)) ||
			    check(cudaMemsetAsync(sched.hist, 0, sizeof(uint32_t) * RDP_SCHED_BUCKETS, stream)))
				return false;
			if (check(rdp_sched_init_weights(&sched, 1u, stream))) return false;
			sched_ready = true;
			generation++;
		}
		sched.order_enabled = order ? 1u : 0u;
		sched.train_enabled = train ? 1u : 0u;
		sched.lr = lr;
		sched.train_stride = stride ? stride : 1u;
		record_cycles = train || cycles_requested;
		return sched_buffers(caps.tile_items) && sched_prim_buffers(caps.prims);
	}

	// While a capture is being recorded, buffers that growth replaces stay allocated: the launches
	// recorded before the growth point into them.  The graph takes them and frees them when it is
	// destroyed.
	std::vector<void *> *retired = nullptr;
	void release(void *p)
	{
		if (!p) return;
		if (retired) retired->push_back(p);
		else cudaFree(p);
	}

	uint32_t sched_prim_capacity = 0;
	bool sched_prim_buffers(uint32_t n)
	{
		if (!sched_ready || n <= sched_prim_capacity) return true;
		release(sched.featbits);
		sched.featbits = nullptr;
		if (check(cudaMalloc(&sched.featbits, sizeof(uint16_t) * size_t(n)))) return false;
		sched_prim_capacity = n;
		generation++;
		return true;
	}

	bool sched_buffers(uint32_t n)
	{
		if (!sched_ready || n <= sched_capacity) return true;
		release(sched.features);
		release(sched.pred);
		release(sched.bucket);
		sched.features = nullptr;
		sched.pred = nullptr;
		sched.bucket = nullptr;
		if (check(cudaMalloc(&sched.features, sizeof(float) * RDP_MLP_IN * size_t(n))) ||
		    check(cudaMalloc(&sched.pred, sizeof(float) * size_t(n))) || check(cudaMalloc(&sched.bucket, 4 * size_t(n))))
			return false;
		sched_capacity = n;
		sched.capacity = n;
		generation++;
		return true;
	}

	void sched_free()
	{
		cudaFree(sched.w16);
		cudaFree(sched.w32);
		cudaFree(sched.adam_m);
		cudaFree(sched.adam_v);
		cudaFree(sched.grad);
		cudaFree(sched.adam_t);
		cudaFree(sched.loss);
		cudaFree(sched.hist);
		cudaFree(sched.cursor);
		cudaFree(sched.featbits);
		cudaFree(sched.features);
		cudaFree(sched.pred);
		cudaFree(sched.bucket);
		sched = RdpSchedDev{};
		sched_ready = false;
		sched_capacity = 0;
		sched_prim_capacity = 0;
	}

	bool check(cudaError_t e)
	{
		if (e != cudaSuccess) failed = true;
		return e != cudaSuccess;
	}

	bool init(int dev, cudaStream_t s)
	{
		device = dev;
		stream = s;
		int sms = 0;
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
		sms = std::max(sms, 1);
		for (int v = 0; v < RDP_SHADE_VARIANTS; v++) shade_ctas_v[v] = uint32_t(sms) * uint32_t(rdp_kernels_shade_ctas_per_sm(v));
		// RDP_BLEND_KERNEL=0|1 selects the blend kernel (look-ahead through registers / staged by bulk
		// copies); the default is the one measured faster on the batched workload.
		if (const char *e = getenv("RDP_BLEND_KERNEL")) blend_kernel = atoi(e) ? 1u : 0u;
		blend_ctas = uint32_t(sms) * uint32_t(rdp_kernels_blend_ctas_per_sm(int(blend_kernel)));
		tuner.active = shade_variant_choice(device) < 0;
		num_queues = uint32_t(sms);
		if (const char *e = getenv("RDP_SHADE_PERM_MIN_PRIMS")) perm_min_prims = uint32_t(strtoul(e, nullptr, 10));
		if (const char *e = getenv("RDP_SHADE_QUEUE_MIN")) queue_min = uint32_t(strtoul(e, nullptr, 10));
		if (const char *e = getenv("RDP_PAIR_CAPACITY")) initial_pairs = std::max(1u, uint32_t(strtoul(e, nullptr, 10)));
		if (const char *e = getenv("RDP_SPAN_ROW_CAPACITY"))
			initial_span_rows = std::max(1u, uint32_t(strtoul(e, nullptr, 10)));
		// RDP_RASTER_PATH=fused: every launch takes the fused per-tile kernel (k_raster: shading and
		// blending in one CTA per tile) instead of the pair path, for comparing the two designs.
		if (const char *e = getenv("RDP_RASTER_PATH"))
			if (!strcmp(e, "fused"))
			{
				fused_only = true;
				initial_pairs = 1;
				initial_span_rows = 1;
			}
		if (const char *e = getenv("RDP_LAUNCH_LOG"))
		{
			launch_log = fopen(e, "a");
			if (launch_log && check(cudaMalloc(&d_launch_pairs, kLaunchLogSlots * 4))) return false;
		}
		if (check(cudaMalloc(&d_ctrl, 64)) || check(cudaMalloc(&d_pair_log, 256 * 4)) ||
		    check(cudaMalloc(&d_queues, queue_bytes())) ||
		    check(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking)) ||
		    check(cudaStreamCreateWithFlags(&side_stream, cudaStreamNonBlocking)) ||
		    check(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming)) ||
		    check(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming)))
			return false;
		for (int k = 0; k < kStagingSlots; k++)
			if (check(cudaEventCreateWithFlags(&slot_copied[k], cudaEventDisableTiming)) ||
			    check(cudaEventCreateWithFlags(&slot_free[k], cudaEventDisableTiming)))
				return false;
		return !check(cudaMemsetAsync(d_ctrl, 0, 64, stream)) && !check(cudaMemsetAsync(d_queues, 0, queue_bytes(), stream));
	}

	int current_variant()
	{
		int v = shade_variant_choice(device);
		return v >= 0 && v < RDP_SHADE_VARIANTS ? v : 0;
	}

	// Appends the pair counts of logged launches whose kernels have finished (the stream is idle).
	void flush_launch_log()
	{
		if (!launch_log || launch_log_pending.empty()) return;
		std::vector<uint32_t> pairs(kLaunchLogSlots);
		if (cudaMemcpy(pairs.data(), d_launch_pairs, 4 * size_t(kLaunchLogSlots), cudaMemcpyDeviceToHost) != cudaSuccess)
		{
			cudaGetLastError();
			return;
		}
		for (auto &e : launch_log_pending) fprintf(launch_log, "launch %llu pairs %u\n", (unsigned long long)e.first, pairs[e.second]);
		fflush(launch_log);
		launch_log_pending.clear();
	}

	// Folds finished tuning samples in (non-blocking for unfinished ones).
	void tune_collect()
	{
		if (tuner.pending.empty()) return;
		uint32_t log[256];
		if (cudaMemcpy(log, d_pair_log, sizeof(log), cudaMemcpyDeviceToHost) != cudaSuccess)
		{
			cudaGetLastError();
			return;
		}
		std::vector<ShadeTuner::Sample> keep;
		for (auto &sm : tuner.pending)
		{
			float ms = 0.0f;
			cudaError_t q = cudaEventQuery(sm.ev[1]);
			if (q == cudaErrorNotReady)
			{
				keep.push_back(sm);
				continue;
			}
			if (q == cudaSuccess && log[sm.slot] != 0xffffffffu && cudaEventElapsedTime(&ms, sm.ev[0], sm.ev[1]) == cudaSuccess)
			{
				tuner.ms[sm.variant] += ms;
				tuner.pairs[sm.variant] += log[sm.slot];
				tuner.count[sm.variant]++;
			}
			cudaGetLastError();
			tuner.pool.push_back(sm.ev[0]);
			tuner.pool.push_back(sm.ev[1]);
		}
		tuner.pending.swap(keep);
	}

	// At a sync point (the stream is idle): ends a tuning epoch; after the last one, keeps
	// the variant with the least k_shade time per pair.
	void tune_epoch()
	{
		flush_launch_log();
		if (!tuner.active) return;
		if (shade_variant_choice(device) >= 0)
		{
			tuner.active = false;
			return;
		}
		tune_collect();
		if (tuner.in_epoch == 0) return; // nothing rasterised since the last sync point
		tuner.in_epoch = 0;
		if (++tuner.epoch < RDP_SHADE_VARIANTS) return;
		int best = -1;
		double best_rate = 0.0;
		for (int v = 0; v < RDP_SHADE_VARIANTS; v++)
		{
			if (tuner.pairs[v] <= 0.0) continue;
			double rate = tuner.ms[v] / tuner.pairs[v];
			if (best < 0 || rate < best_rate)
			{
				best = v;
				best_rate = rate;
			}
		}
		if (best < 0) best = 0;
		tuner.active = false;
		if (shade_variant_choice(device) < 0) shade_variant_choice(device) = best;
	}

	void free_all()
	{
		cudaFree(d_geom);
		cudaFree(d_attr);
		cudaFree(d_shade);
		cudaFree(d_masks);
		cudaFree(d_tmem_keep);
		cudaFree(d_tile_counts);
		cudaFree(d_pair_offsets);
		cudaFree(d_tile_order);
		cudaFree(d_tile_cycles);
		cudaFree(d_nonempty);
		cudaFree(d_scan_blocks);
		cudaFree(d_prim_pairs);
		cudaFree(d_prim_offsets);
		cudaFree(d_prim_blocks);
		cudaFree(d_prim_rows);
		cudaFree(d_spans);
		cudaFree(d_shade_list);
		cudaFree(d_pairs);
		cudaFree(d_scratch);
		cudaFree(d_staging);
		d_geom = nullptr;
		d_attr = nullptr;
		d_shade = nullptr;
		d_masks = d_tmem_keep = d_tile_counts = d_pair_offsets = d_tile_order = d_tile_cycles = d_nonempty = nullptr;
		d_scan_blocks = nullptr;
		d_prim_pairs = d_prim_offsets = d_prim_blocks = d_prim_rows = nullptr;
		d_spans = nullptr;
		d_shade_list = nullptr;
		d_pairs = nullptr;
		d_scratch = nullptr;
		d_staging = nullptr;
	}

	void destroy()
	{
		if (stream) cudaStreamSynchronize(stream);
		if (copy_stream) cudaStreamSynchronize(copy_stream);
		free_all();
		sched_free();
		cudaFree(d_ctrl);
		if (launch_log)
		{
			if (stream) cudaStreamSynchronize(stream);
			flush_launch_log();
			fclose(launch_log);
			launch_log = nullptr;
		}
		cudaFree(d_launch_pairs);
		d_launch_pairs = nullptr;
		cudaFree(d_pair_log);
		cudaFree(d_queues);
		d_ctrl = nullptr;
		d_pair_log = nullptr;
		d_queues = nullptr;
		for (int k = 0; k < kStagingSlots; k++)
		{
			if (slot_copied[k]) cudaEventDestroy(slot_copied[k]);
			if (slot_free[k]) cudaEventDestroy(slot_free[k]);
			slot_copied[k] = slot_free[k] = nullptr;
		}
		if (copy_stream) cudaStreamDestroy(copy_stream);
		copy_stream = nullptr;
		if (side_stream)
		{
			cudaStreamSynchronize(side_stream);
			cudaStreamDestroy(side_stream);
		}
		side_stream = nullptr;
		if (fork_ev) cudaEventDestroy(fork_ev);
		if (join_ev) cudaEventDestroy(join_ev);
		fork_ev = join_ev = nullptr;
		tuner.destroy();
		for (auto &st : staging)
		{
			if (st.h) cudaFreeHost(st.h);
			if (st.done) cudaEventDestroy(st.done);
		}
		staging.clear();
	}

	// Grows the buffers to hold `need`.  Called with the stream idle.
	bool ensure(const ExecCaps &need)
	{
		bool grow_prims = need.prims > caps.prims, grow_tiles = need.tile_items > caps.tile_items;
		bool grow_passes = need.passes > caps.passes, grow_pairs = need.pairs > caps.pairs;
		bool grow_staging = need.staging > caps.staging, grow_spans = need.span_rows > caps.span_rows;
		bool grow_uploads = need.uploads > caps.uploads, grow_masks = need.mask_words > caps.mask_words;
		if (!(grow_prims || grow_tiles || grow_passes || grow_pairs || grow_staging || grow_spans || grow_uploads ||
		      grow_masks))
			return true;
		if (check(cudaStreamSynchronize(stream)) || (copy_stream && check(cudaStreamSynchronize(copy_stream))))
			return false;
		for (auto &st : staging) st.in_flight = false;
		generation++;
		if (grow_prims)
		{
			uint32_t n = std::max(need.prims, caps.prims * 2);
			release(d_geom);
			release(d_attr);
			release(d_shade);
			release(d_prim_pairs);
			release(d_prim_offsets);
			release(d_prim_blocks);
			release(d_prim_rows);
			d_geom = nullptr;
			d_attr = nullptr;
			d_shade = nullptr;
			d_prim_pairs = d_prim_offsets = d_prim_blocks = d_prim_rows = nullptr;
			if (check(cudaMalloc(&d_geom, sizeof(RdpPrimGeom) * n)) || check(cudaMalloc(&d_attr, sizeof(RdpPrimAttr) * n)) ||
			    check(cudaMalloc(&d_shade, sizeof(RdpPrimShade) * n)) || check(cudaMalloc(&d_prim_pairs, size_t(n) * 4)) ||
			    check(cudaMalloc(&d_prim_offsets, size_t(n) * 4)) || check(cudaMalloc(&d_prim_rows, size_t(n) * 4)) ||
			    check(cudaMalloc(&d_prim_blocks, (size_t(n) / 1024 + 2) * 8)))
				return false;
			caps.prims = n;
			if (!sched_prim_buffers(n)) return false;
		}
		if (grow_tiles)
		{
			uint32_t n = std::max(need.tile_items, caps.tile_items + caps.tile_items / 2);
			release(d_tile_counts);
			release(d_pair_offsets);
			release(d_tile_order);
			release(d_tile_cycles);
			release(d_nonempty);
			release(d_scan_blocks);
			d_tile_counts = d_pair_offsets = d_tile_order = d_tile_cycles = d_nonempty = d_scan_blocks = nullptr;
			if (check(cudaMalloc(&d_tile_counts, size_t(n + 1) * 4)) || check(cudaMalloc(&d_pair_offsets, size_t(n + 1) * 4)) ||
			    check(cudaMalloc(&d_tile_order, size_t(n) * 4)) || check(cudaMalloc(&d_tile_cycles, size_t(n) * 4)) ||
			    check(cudaMalloc(&d_nonempty, size_t(n) * 4)) ||
			    check(cudaMalloc(&d_scan_blocks, (size_t(n) / 1024 + 2) * 8)))
				return false;
			// Counts are self-clearing between launches; they start at zero.
			if (check(cudaMemsetAsync(d_tile_counts, 0, size_t(n + 1) * 4, stream))) return false;
			caps.tile_items = n;
			if (!sched_buffers(n)) return false;
		}
		if (grow_masks)
		{
			// The tiles' primitive bitmasks, laid out per launch (each pass's tiles with its own word
			// count); self-clearing between launches, so they start at zero.
			size_t n = std::max(need.mask_words, caps.mask_words + caps.mask_words / 2);
			release(d_masks);
			d_masks = nullptr;
			if (check(cudaMalloc(&d_masks, n * 4)) || check(cudaMemsetAsync(d_masks, 0, n * 4, stream))) return false;
			caps.mask_words = n;
		}
		if (grow_passes) caps.passes = std::max(need.passes, caps.passes * 2);
		if (grow_uploads)
		{
			uint32_t n = std::max(need.uploads, caps.uploads + caps.uploads / 2);
			release(d_tmem_keep);
			d_tmem_keep = nullptr;
			if (check(cudaMalloc(&d_tmem_keep, size_t(n) * 64 * 4))) return false;
			caps.uploads = n;
		}
		if (grow_pairs)
		{
			uint32_t n = std::max(need.pairs, caps.pairs * 2);
			release(d_pairs);
			release(d_shade_list);
			release(d_scratch);
			d_pairs = nullptr;
			d_shade_list = nullptr;
			d_scratch = nullptr;
			if (check(cudaMalloc(&d_pairs, size_t(n) * sizeof(uint2))) || check(cudaMalloc(&d_shade_list, size_t(n) * sizeof(uint4))) ||
			    check(cudaMalloc(&d_scratch, size_t(n) * 64 * sizeof(uint2))))
				return false;
			caps.pairs = n;
		}
		if (grow_spans)
		{
			uint32_t n = std::max(need.span_rows, caps.span_rows + caps.span_rows / 2);
			release(d_spans);
			d_spans = nullptr;
			if (check(cudaMalloc(&d_spans, size_t(n) * RDP_SPAN_ROW_BYTES))) return false;
			caps.span_rows = n;
		}
		if (grow_staging)
		{
			size_t n = std::max(need.staging, caps.staging + caps.staging / 2);
			release(d_staging);
			d_staging = nullptr;
			if (check(cudaMalloc(&d_staging, kStagingSlots * n))) return false;
			caps.staging = n;
		}
		return !check(cudaStreamSynchronize(stream));
	}

	// With the stream idle: the device error word (ctrl[8]; bit 0: a k_blend staging wait gave
	// up), cleared once read.  A non-zero word means a launch's results are incomplete.
	uint32_t take_device_error()
	{
		uint32_t e = 0;
		if (check(cudaMemcpy(&e, d_ctrl + 8, 4, cudaMemcpyDeviceToHost))) return ~0u;
		if (e && check(cudaMemset(d_ctrl + 8, 0, 4))) return ~0u;
		if (e) failed = true;
		return e;
	}

	// With the stream idle: grows the pair scratch and the span rows to the largest counts a
	// launch has needed, so that later launches take the pair path instead of the fused fallback.
	bool adapt_pairs()
	{
		if (fused_only) return true;
		uint32_t seen[6] = { 0, 0, 0, 0, 0, 0 };
		if (check(cudaMemcpy(seen, d_ctrl, sizeof(seen), cudaMemcpyDeviceToHost))) return false;
		if (seen[2] <= caps.pairs && seen[5] <= caps.span_rows) return true;
		ExecCaps need = caps;
		if (seen[2] > caps.pairs)
		{
			need.pairs = 1u;
			while (need.pairs < seen[2] && need.pairs < (1u << 30)) need.pairs <<= 1;
		}
		if (seen[5] > caps.span_rows)
		{
			need.span_rows = 1u;
			while (need.span_rows < seen[5] && need.span_rows < (1u << 30)) need.span_rows <<= 1;
		}
		return ensure(need);
	}

	static size_t staging_bytes_for(const PassView *v, uint32_t n)
	{
		size_t b = align16(sizeof(RdpPass) * kMaxTargets * n) + align16(4 * n) + 256;
		for (uint32_t i = 0; i < n; i++)
			b += align16(sizeof(RdpPrimIn) * v[i].num_prims) + align16(4 * v[i].num_words) +
			     align16(4 * RDP_STATE_BLOCK_WORDS * v[i].num_state_blocks) + align16(sizeof(RdpTile) * 8 * v[i].num_tilesets) +
			     align16(sizeof(RdpUpload) * v[i].num_uploads);
		return b;
	}

	// Launches the kernel chain once for the passes v[0..n) (distinct instances).
	// With `cap`, the launch is recorded with device-resident inputs instead.
	// `upscaled`: the views are upscaled passes (RdpPass.scale), rendered by k_raster_upscaled.
	bool launch(const PassView *v, uint32_t n, CaptureSink *cap, bool upscaled = false)
	{
		if (!n || failed) return !failed;
		ExecCaps need = caps;
		uint32_t prims = 0, tiles = 0, descs = 0, uploads = 0;
		size_t mask_words = 0;
		for (uint32_t i = 0; i < n; i++)
		{
			prims += v[i].num_prims;
			uploads += v[i].num_uploads;
			descs += v[i].num_targets;
			for (uint32_t t = 0; t < v[i].num_targets; t++)
			{
				const uint32_t tt = v[i].target[t].tiles_x * v[i].target[t].tiles_y;
				tiles += tt;
				mask_words += size_t(tt) * RDP_MASK_WORDS(v[i].target_prims[t]);
			}
		}
		need.passes = std::max(need.passes, n);
		need.descs = std::max(need.descs, descs);
		need.prims = std::max(need.prims, std::max(prims, 1u));
		need.uploads = std::max(need.uploads, std::max(uploads, 1u));
		need.mask_words = std::max(need.mask_words, std::max<size_t>(mask_words, 1));
		need.tile_items = std::max(need.tile_items, std::max(tiles, 1u));
		need.pairs = std::max(need.pairs, initial_pairs);
		need.span_rows = std::max(need.span_rows, initial_span_rows);
		need.staging = std::max(need.staging, staging_bytes_for(v, n));
		retired = cap ? &cap->buffers : nullptr;
		const bool grown = ensure(need);
		retired = nullptr;
		if (!grown) return false;

		Staging *stp = take_staging(staging_bytes_for(v, n));
		if (!stp) return false;
		Staging &st = *stp;
		uint8_t *h = st.h;
		size_t off = 0;
		auto reserve = [&](size_t bytes) -> size_t {
			size_t at = off;
			off = align16(off + bytes);
			return at;
		};
		uint32_t num_descs = 0;
		for (uint32_t i = 0; i < n; i++) num_descs += v[i].num_targets;
		size_t o_pass = reserve(sizeof(RdpPass) * num_descs);
		size_t o_list = reserve(8 * n); // TMEM passes in launch order, then largest first
		RdpPass *passes = reinterpret_cast<RdpPass *>(h + o_pass);
		uint32_t *tmem_list = reinterpret_cast<uint32_t *>(h + o_list);
		uint32_t num_tmem = 0;
		uint32_t prim_base = 0, word_base = 0, sb_base = 0, ts_base = 0, up_base = 0, tile_base = 0;
		size_t mask_base = 0;
		// Sections: all prims, then all words, state blocks, tile sets, uploads; each view's
		// share of a section is contiguous.  The views are copied in parallel.
		std::vector<size_t> at(size_t(n) * 5);
		size_t cursor = off;
		size_t o_prims = cursor;
		for (uint32_t i = 0; i < n; i++) at[i * 5 + 0] = cursor, cursor += sizeof(RdpPrimIn) * v[i].num_prims;
		cursor = align16(cursor);
		size_t o_words = cursor;
		for (uint32_t i = 0; i < n; i++) at[i * 5 + 1] = cursor, cursor += 4 * size_t(v[i].num_words);
		cursor = align16(cursor);
		size_t o_sb = cursor;
		for (uint32_t i = 0; i < n; i++)
			at[i * 5 + 2] = cursor, cursor += 4 * size_t(RDP_STATE_BLOCK_WORDS) * v[i].num_state_blocks;
		cursor = align16(cursor);
		size_t o_ts = cursor;
		for (uint32_t i = 0; i < n; i++) at[i * 5 + 3] = cursor, cursor += sizeof(RdpTile) * 8 * v[i].num_tilesets;
		cursor = align16(cursor);
		size_t o_up = cursor;
		for (uint32_t i = 0; i < n; i++) at[i * 5 + 4] = cursor, cursor += sizeof(RdpUpload) * v[i].num_uploads;
		auto fill = [&](uint32_t i) {
			memcpy(h + at[i * 5 + 0], v[i].prims, sizeof(RdpPrimIn) * v[i].num_prims);
			memcpy(h + at[i * 5 + 1], v[i].words, 4 * size_t(v[i].num_words));
			memcpy(h + at[i * 5 + 2], v[i].state_blocks, 4 * size_t(RDP_STATE_BLOCK_WORDS) * v[i].num_state_blocks);
			memcpy(h + at[i * 5 + 3], v[i].tilesets, sizeof(RdpTile) * 8 * v[i].num_tilesets);
			memcpy(h + at[i * 5 + 4], v[i].uploads, sizeof(RdpUpload) * v[i].num_uploads);
		};
		if (cursor - o_prims >= kParallelFillBytes) pool.run(n, fill);
		else
			for (uint32_t i = 0; i < n; i++) fill(i);
		off = align16(cursor) + 16;
		uint32_t d = 0;
		for (uint32_t i = 0; i < n; i++)
		{
			for (uint32_t t = 0; t < v[i].num_targets; t++, d++)
			{
				RdpPass p = v[i].target[t];
				p.prim_begin = prim_base;
				p.prim_count = v[i].target_prims[t];
				p.word_base = word_base;
				p.sb_base = sb_base;
				p.ts_base = ts_base;
				p.upload_begin = up_base;
				p.upload_count = t == 0 ? v[i].num_uploads : 0;
				p.tile_item_begin = tile_base;
				p.mask_words = RDP_MASK_WORDS(p.prim_count);
				p.masks = d_masks + mask_base;
				passes[d] = p;
				if (t == 0 && v[i].num_uploads) tmem_list[num_tmem++] = d;
				prim_base += p.prim_count;
				tile_base += p.tiles_x * p.tiles_y;
				mask_base += size_t(p.tiles_x) * p.tiles_y * p.mask_words;
			}
			word_base += v[i].num_words;
			sb_base += v[i].num_state_blocks;
			ts_base += v[i].num_tilesets;
			up_base += v[i].num_uploads;
		}

		// The carry kernel takes the TMEM passes with the most uploads first (their CTAs run longest).
		uint32_t *carry_list = tmem_list + n;
		std::copy(tmem_list, tmem_list + num_tmem, carry_list);
		std::stable_sort(carry_list, carry_list + num_tmem, [&](uint32_t a, uint32_t b) {
			return passes[a].upload_count > passes[b].upload_count;
		});
		const int slot = staging_slot;
		uint8_t *dst = d_staging + size_t(slot) * caps.staging;
		if (cap)
		{
			if (check(cudaMalloc(&dst, off))) return false;
			cap->buffers.push_back(dst);
			if (check(cudaMemcpy(dst, h, off, cudaMemcpyHostToDevice))) return false;
		}
		else
		{
			staging_slot = (staging_slot + 1) % kStagingSlots;
			if (check(cudaStreamWaitEvent(copy_stream, slot_free[slot], 0)) ||
			    check(cudaMemcpyAsync(dst, h, off, cudaMemcpyHostToDevice, copy_stream)) ||
			    check(cudaEventRecord(st.done, copy_stream)) || check(cudaEventRecord(slot_copied[slot], copy_stream)) ||
			    check(cudaStreamWaitEvent(stream, slot_copied[slot], 0)))
				return false;
			st.in_flight = true;
		}
		staging_bytes += off;

		RdpLaunch L = {};
		L.prims_in = reinterpret_cast<const RdpPrimIn *>(dst + o_prims);
		L.num_prims = prim_base;
		L.words = reinterpret_cast<const uint32_t *>(dst + o_words);
		L.state_blocks = reinterpret_cast<const uint32_t *>(dst + o_sb);
		L.passes = reinterpret_cast<const RdpPass *>(dst + o_pass);
		L.num_passes = num_descs;
		L.geom = d_geom;
		L.attr = d_attr;
		L.shade = d_shade;
		L.tilesets = reinterpret_cast<const RdpTile *>(dst + o_ts);
		L.tmem_pass_list = reinterpret_cast<const uint32_t *>(dst + o_list);
		L.tmem_carry_list = L.tmem_pass_list + n;
		L.num_tmem_passes = num_tmem;
		L.uploads = reinterpret_cast<const RdpUpload *>(dst + o_up);
		L.num_uploads = up_base;
		L.tmem_keep = d_tmem_keep;
		L.tile_counts = d_tile_counts;
		L.nonempty_tiles = d_nonempty;
		L.scan_blocks = d_scan_blocks;
		L.pair_offsets = d_pair_offsets;
		L.pairs = d_pairs;
		L.ctrl = d_ctrl;
		L.pair_capacity = caps.pairs;
		// k_shade work order (process-wide per device): 0 = fixed stride over the pairs in tile
		// order, 1 = per-SM queues over tile order, 2 = per-SM queues over primitive-major order
		// for launches of at least perm_min_prims primitives (smaller ones gain less from it than
		// the primitive scan costs), else as 1.
		const int shade_order = shade_order_choice(device);
		L.shade_queues = shade_order >= 1 ? d_queues : nullptr;
		L.num_shade_queues = shade_order >= 1 ? num_queues : 0u;
		L.shade_queue_min = queue_min;
		L.shade_list = shade_order == 2 && prim_base >= perm_min_prims ? d_shade_list : nullptr;
		L.prim_pairs = d_prim_pairs;
		L.prim_offsets = d_prim_offsets;
		L.prim_scan_blocks = d_prim_blocks;
		L.upscaled = upscaled ? 1u : 0u;
		// Launches whose passes only fill rectangles (a frame's clears) take the per-tile fill kernel.
		bool fill_only = !upscaled && tile_base != 0;
		for (uint32_t i = 0; i < n && fill_only; i++) fill_only = v[i].fill_only;
		L.fill_only = fill_only ? 1u : 0u;
		L.side_stream = side_stream;
		L.fork_event = fork_ev;
		L.join_event = join_ev;
		int variant = current_variant();
		bool sample = false;
		if (!upscaled && !fill_only && tuner.active && shade_variant_choice(device) < 0 && !cap && tile_base &&
		    tuner.in_epoch < ShadeTuner::kMaxSamplesPerEpoch)
		{
			variant = int((tuner.in_epoch + uint32_t(tuner.epoch)) % RDP_SHADE_VARIANTS);
			tuner.in_epoch++;
			sample = true;
		}
		L.shade_variant = uint32_t(variant);
		L.shade_ctas = shade_ctas_v[variant];
		L.blend_ctas = blend_ctas;
		L.blend_kernel = blend_kernel;
		L.pair_log = sample ? d_pair_log : nullptr;
		L.log_slot = sample ? uint32_t(tuner.samples_taken++ % 256) : 0u;
		if (!upscaled && !fill_only && !sample && !cap && launch_log && tile_base && launch_log_pending.size() < kLaunchLogSlots)
		{
			L.pair_log = d_launch_pairs;
			L.log_slot = uint32_t(launch_log_pending.size());
			launch_log_pending.emplace_back(launches, L.log_slot);
		}
		L.spans = d_spans;
		L.span_capacity = caps.span_rows;
		L.prim_rows = d_prim_rows;
		L.num_sms = num_queues;
		L.scratch = d_scratch;
		L.num_tile_items = tile_base;
		L.tile_cycles = record_cycles ? d_tile_cycles : nullptr;
		L.tile_order = nullptr;
		if (!upscaled && !fill_only && sched_ready && (sched.order_enabled || sched.train_enabled))
		{
			sched.order = d_tile_order;
			L.sched = &sched;
		}
		launches++;
		if (cap)
		{
			for (auto &e : L.shade_events)
				if (check(cudaEventCreate(&e))) return false;
			for (auto &e : L.blend_events)
				if (check(cudaEventCreate(&e))) return false;
			cap->launches.push_back(L);
			return true;
		}
		if (sample)
		{
			ShadeTuner::Sample sm;
			sm.variant = variant;
			sm.ev[0] = tuner.event();
			sm.ev[1] = tuner.event();
			sm.slot = L.log_slot;
			L.shade_events[0] = sm.ev[0];
			L.shade_events[1] = sm.ev[1];
			tuner.pending.push_back(sm);
		}
		if (check(rdp_kernels_launch(&L, stream)) || check(cudaEventRecord(slot_free[slot], stream))) return false;
		kernel_launches += rdp_kernels_count(&L);
		return true;
	}
};

} // namespace rdpx

#endif
