/*
 * Learned tile scheduling (see sched.h): feature extraction, MLP inference, bucket sort of the
 * k_blend queue, and the training kernels (forward + backward + Adam), all for sm_103a.
 *
 * One warp evaluates one sample: lane l owns hidden units l and l + 32 of each layer.  Weights
 * live in shared memory as FP32 copies of the FP16 parameters, transposed where that keeps the
 * lanes' accesses on consecutive banks.
 */
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include "sched.h"

namespace rdpsched {

constexpr int H = RDP_MLP_HIDDEN, IN = RDP_MLP_IN;
constexpr int WARPS = 8;

// Shared-memory copy of the network for the forward pass.
struct NetS
{
	float w1t[IN * H]; // [k][j]
	float b1[H];
	float w2t[H * H];  // [j][i] = W2[i][j]
	float b2[H];
	float w3[H];
	float b3;
};

__device__ void load_net(NetS &n, const __half *__restrict__ w)
{
	for (int p = threadIdx.x; p < H * IN; p += blockDim.x)
	{
		int j = p / IN, k = p % IN;
		n.w1t[k * H + j] = __half2float(w[RDP_MLP_W1 + p]);
	}
	for (int p = threadIdx.x; p < H * H; p += blockDim.x)
	{
		int i = p / H, j = p % H;
		n.w2t[j * H + i] = __half2float(w[RDP_MLP_W2 + p]);
	}
	for (int p = threadIdx.x; p < H; p += blockDim.x)
	{
		n.b1[p] = __half2float(w[RDP_MLP_B1 + p]);
		n.b2[p] = __half2float(w[RDP_MLP_B2 + p]);
		n.w3[p] = __half2float(w[RDP_MLP_W3 + p]);
	}
	if (threadIdx.x == 0) n.b3 = __half2float(w[RDP_MLP_B3]);
}

// Forward pass of one sample by one warp; x, h1, h2 are the warp's shared scratch.
__device__ float warp_forward(const NetS &n, const float *x, float *h1, float *h2, int lane)
{
#pragma unroll
	for (int r = 0; r < 2; r++)
	{
		int j = lane + 32 * r;
		float acc = n.b1[j];
#pragma unroll
		for (int k = 0; k < IN; k++) acc = fmaf(n.w1t[k * H + j], x[k], acc);
		h1[j] = fmaxf(acc, 0.0f);
	}
	__syncwarp();
	float part = 0.0f;
#pragma unroll
	for (int r = 0; r < 2; r++)
	{
		int i = lane + 32 * r;
		float acc = n.b2[i];
		for (int j = 0; j < H; j++) acc = fmaf(n.w2t[j * H + i], h1[j], acc);
		acc = fmaxf(acc, 0.0f);
		h2[i] = acc;
		part = fmaf(n.w3[i], acc, part);
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
	__syncwarp();
	return part + n.b3;
}

// ------------------------------------------------------------------ scheduling
// Adds `count` lanes' worth of `b` to counter[b] with one atomic per distinct value in the warp
// (most tiles share the last bucket); returns each lane's position among its peers' slots.
__device__ __forceinline__ uint32_t warp_aggregated_add(uint32_t *counter, uint32_t b, bool active)
{
	const unsigned mask = __ballot_sync(0xffffffffu, active);
	uint32_t pos = 0;
	if (active)
	{
		const int lane = threadIdx.x & 31;
		const unsigned peers = __match_any_sync(mask, b);
		const int leader = __ffs(peers) - 1;
		uint32_t base = 0;
		if (lane == leader) base = atomicAdd(&counter[b], uint32_t(__popc(peers)));
		base = __shfl_sync(peers, base, leader);
		pos = base + uint32_t(__popc(peers & ((1u << lane) - 1u)));
	}
	return pos;
}

// Per non-empty tile: prediction from the features k_expand wrote, bucket (descending cost).
// A warp looks at 32 tiles at a time and evaluates the network only for those with enough pairs.
__global__ void __launch_bounds__(WARPS * 32) k_tile_predict(RdpSchedDev s, const uint32_t *__restrict__ offsets,
                                                             const uint32_t *__restrict__ ctrl,
                                                             const uint32_t *__restrict__ nonempty)
{
	__shared__ NetS net;
	__shared__ float s_x[WARPS][IN], s_h1[WARPS][H], s_h2[WARPS][H];
	if (ctrl[1]) return;
	load_net(net, s.w16);
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t n = ctrl[3];
	for (uint32_t base = (blockIdx.x * WARPS + warp) * 32u; base < n; base += gridDim.x * WARPS * 32u)
	{
		const uint32_t k = base + uint32_t(lane);
		const bool valid = k < n;
		const uint32_t item = valid ? nonempty[k] : 0u;
		const uint32_t np = valid ? offsets[item + 1] - offsets[item] : 0u;
		float pred = 0.0f;
		uint32_t b = RDP_SCHED_BUCKETS - 1;
		unsigned todo = __ballot_sync(0xffffffffu, valid && np >= RDP_SCHED_MIN_PAIRS);
		while (todo)
		{
			const int src = __ffs(todo) - 1;
			todo &= todo - 1;
			const uint32_t it = __shfl_sync(0xffffffffu, item, src);
			if (lane < IN) s_x[warp][lane] = s.features[size_t(it) * IN + lane];
			__syncwarp();
			const float p = warp_forward(net, s_x[warp], s_h1[warp], s_h2[warp], lane);
			if (lane == src)
			{
				pred = p;
				int bb = int((2.0f - p) * (RDP_SCHED_BUCKETS / 2));
				b = uint32_t(bb < 0 ? 0 : (bb >= RDP_SCHED_BUCKETS - 1 ? RDP_SCHED_BUCKETS - 2 : bb));
			}
		}
		if (valid)
		{
			s.pred[k] = pred;
			s.bucket[k] = b;
		}
		warp_aggregated_add(s.hist, b, valid);
	}
}

// Single CTA: bucket counts -> write cursors (exclusive scan); clears the counts.
__global__ void __launch_bounds__(RDP_SCHED_BUCKETS) k_bucket_scan(RdpSchedDev s, const uint32_t *__restrict__ ctrl)
{
	__shared__ uint32_t warp_sums[32];
	if (ctrl[1]) return;
	const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
	uint32_t v = s.hist[t], x = v;
	s.hist[t] = 0u;
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
		uint32_t w = warp_sums[lane];
#pragma unroll
		for (int o = 1; o < 32; o <<= 1)
		{
			uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
			if (lane >= o) w += y;
		}
		warp_sums[lane] = w;
	}
	__syncthreads();
	s.cursor[t] = (wid ? warp_sums[wid - 1] : 0u) + x - v;
}

__global__ void k_bucket_scatter(RdpSchedDev s, const uint32_t *__restrict__ ctrl, const uint32_t *__restrict__ nonempty)
{
	if (ctrl[1]) return;
	const uint32_t n = ctrl[3];
	const uint32_t stride = gridDim.x * blockDim.x;
	for (uint32_t k0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); k0 < n; k0 += stride)
	{
		const uint32_t k = k0 + (threadIdx.x & 31u);
		const bool valid = k < n;
		const uint32_t b = valid ? s.bucket[k] : 0u;
		const uint32_t pos = warp_aggregated_add(s.cursor, b, valid);
		if (valid) s.order[pos] = nonempty[k];
	}
}

// ------------------------------------------------------------------ training
// Shared-memory layout of the gradient kernel (dynamic): the forward net, W2 row-major for
// the backward pass, gradient accumulators (transposed like the weights), per-warp scratch.
struct GradS
{
	NetS net;
	float w2[H * H]; // [i][j]
	float g_w1t[IN * H], g_b1[H], g_w2t[H * H], g_b2[H], g_w3[H], g_b3;
	float x[WARPS][IN], h1[WARPS][H], h2[WARPS][H], dh2[WARPS][H];
};

// Samples: features[k] with target targets[k] (or, when targets is null, log2(1 + cycles of
// tile nonempty[k]) / 16, taking every `stride`-th non-empty tile of the launch).
__global__ void __launch_bounds__(WARPS * 32) k_mlp_grad(const __half *__restrict__ w16, const float *__restrict__ features,
                                                         const float *__restrict__ targets, uint32_t n_fixed,
                                                         const uint32_t *__restrict__ ctrl,
                                                         const uint32_t *__restrict__ nonempty,
                                                         const uint32_t *__restrict__ cycles, uint32_t stride,
                                                         float *__restrict__ grads, float *__restrict__ loss)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	GradS &S = *reinterpret_cast<GradS *>(smem_raw);
	if (ctrl && ctrl[1]) return;
	load_net(S.net, w16);
	for (int p = threadIdx.x; p < H * H; p += blockDim.x) S.w2[p] = __half2float(w16[RDP_MLP_W2 + p]);
	for (int p = threadIdx.x; p < IN * H; p += blockDim.x) S.g_w1t[p] = 0.0f;
	for (int p = threadIdx.x; p < H * H; p += blockDim.x) S.g_w2t[p] = 0.0f;
	for (int p = threadIdx.x; p < H; p += blockDim.x)
	{
		S.g_b1[p] = 0.0f;
		S.g_b2[p] = 0.0f;
		S.g_w3[p] = 0.0f;
	}
	if (threadIdx.x == 0) S.g_b3 = 0.0f;
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t total = targets ? n_fixed : (ctrl[3] + stride - 1) / stride;
	const float scale = total ? 2.0f / float(total) : 0.0f;
	float sq = 0.0f;
	for (uint32_t si = blockIdx.x * WARPS + warp; si < total; si += gridDim.x * WARPS)
	{
		// Fixed samples are rows of `features`; launch samples are non-empty tiles (features by item).
		const uint32_t k = targets ? si : nonempty[si * stride];
		float y;
		if (targets) y = targets[k];
		else y = log2f(1.0f + float(cycles[k])) * (1.0f / 16.0f);
		if (lane < IN) S.x[warp][lane] = features[size_t(k) * IN + lane];
		__syncwarp();
		const float out = warp_forward(S.net, S.x[warp], S.h1[warp], S.h2[warp], lane);
		const float err = out - y;
		if (lane == 0) sq += err * err;
		const float d_out = scale * err;
		// Output layer and the second hidden layer.
#pragma unroll
		for (int r = 0; r < 2; r++)
		{
			const int i = lane + 32 * r;
			const float h2 = S.h2[warp][i];
			atomicAdd(&S.g_w3[i], d_out * h2);
			const float dh2 = h2 > 0.0f ? d_out * S.net.w3[i] : 0.0f;
			S.dh2[warp][i] = dh2;
			atomicAdd(&S.g_b2[i], dh2);
			if (dh2 != 0.0f)
				for (int j = 0; j < H; j++) atomicAdd(&S.g_w2t[j * H + i], dh2 * S.h1[warp][j]);
		}
		if (lane == 0) atomicAdd(&S.g_b3, d_out);
		__syncwarp();
		// First hidden layer.
#pragma unroll
		for (int r = 0; r < 2; r++)
		{
			const int j = lane + 32 * r;
			float acc = 0.0f;
			for (int i = 0; i < H; i++) acc = fmaf(S.dh2[warp][i], S.w2[i * H + j], acc);
			const float dh1 = S.h1[warp][j] > 0.0f ? acc : 0.0f;
			atomicAdd(&S.g_b1[j], dh1);
			if (dh1 != 0.0f)
#pragma unroll
				for (int kk = 0; kk < IN; kk++) atomicAdd(&S.g_w1t[kk * H + j], dh1 * S.x[warp][kk]);
		}
		__syncwarp();
	}
	if (lane == 0 && sq != 0.0f) atomicAdd(&loss[0], sq);
	if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&loss[1], float(total));
	__syncthreads();
	for (int p = threadIdx.x; p < H * IN; p += blockDim.x)
	{
		int j = p / IN, k = p % IN;
		atomicAdd(&grads[RDP_MLP_W1 + p], S.g_w1t[k * H + j]);
	}
	for (int p = threadIdx.x; p < H * H; p += blockDim.x)
	{
		int i = p / H, j = p % H;
		atomicAdd(&grads[RDP_MLP_W2 + p], S.g_w2t[j * H + i]);
	}
	for (int p = threadIdx.x; p < H; p += blockDim.x)
	{
		atomicAdd(&grads[RDP_MLP_B1 + p], S.g_b1[p]);
		atomicAdd(&grads[RDP_MLP_B2 + p], S.g_b2[p]);
		atomicAdd(&grads[RDP_MLP_W3 + p], S.g_w3[p]);
	}
	if (threadIdx.x == 0) atomicAdd(&grads[RDP_MLP_B3], S.g_b3);
}

// Adam on the FP32 master weights; refreshes the FP16 copy and clears the gradients.
__global__ void k_mlp_adam(RdpSchedDev s)
{
	__shared__ float s_t;
	if (threadIdx.x == 0) s_t = float(*s.adam_t + 1u);
	__syncthreads();
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	const float c1 = 1.0f - powf(b1, s_t), c2 = 1.0f - powf(b2, s_t);
	for (int p = threadIdx.x; p < RDP_MLP_PARAMS; p += blockDim.x)
	{
		const float g = s.grad[p];
		const float m = b1 * s.adam_m[p] + (1.0f - b1) * g;
		const float v = b2 * s.adam_v[p] + (1.0f - b2) * g * g;
		s.adam_m[p] = m;
		s.adam_v[p] = v;
		const float w = s.w32[p] - s.lr * (m / c1) / (sqrtf(v / c2) + eps);
		s.w32[p] = w;
		s.w16[p] = __float2half_rn(w);
		s.grad[p] = 0.0f;
	}
	__syncthreads();
	if (threadIdx.x == 0) *s.adam_t += 1u;
}

__global__ void k_loss_clear(float *loss)
{
	loss[0] = 0.0f;
	loss[1] = 0.0f;
}

__global__ void __launch_bounds__(WARPS * 32) k_mlp_forward(const __half *__restrict__ w16, const float *__restrict__ features,
                                                            uint32_t n, float *__restrict__ out)
{
	__shared__ NetS net;
	__shared__ float s_x[WARPS][IN], s_h1[WARPS][H], s_h2[WARPS][H];
	load_net(net, w16);
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (uint32_t k = blockIdx.x * WARPS + warp; k < n; k += gridDim.x * WARPS)
	{
		if (lane < IN) s_x[warp][lane] = features[size_t(k) * IN + lane];
		__syncwarp();
		const float o = warp_forward(net, s_x[warp], s_h1[warp], s_h2[warp], lane);
		if (lane == 0) out[k] = o;
		__syncwarp();
	}
}

// Deterministic initialisation: uniform in +-sqrt(6 / (fan_in + fan_out)) (Glorot), biases 0,
// from a 32-bit integer hash of (seed, parameter index).
__global__ void k_mlp_init(RdpSchedDev s, uint32_t seed)
{
	for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < RDP_MLP_PARAMS; p += gridDim.x * blockDim.x)
	{
		uint32_t h = seed * 0x9E3779B1u ^ uint32_t(p) * 0x85EBCA77u;
		h ^= h >> 15;
		h *= 0x2C1B3C6Du;
		h ^= h >> 12;
		h *= 0x297A2D39u;
		h ^= h >> 15;
		const float u = float(h >> 8) * (1.0f / 16777216.0f) * 2.0f - 1.0f;
		float bound = 0.0f;
		if (p < RDP_MLP_B1) bound = 0.2795f;           // sqrt(6 / (16 + 64))
		else if (p >= RDP_MLP_W2 && p < RDP_MLP_B2) bound = 0.2165f; // sqrt(6 / 128)
		else if (p >= RDP_MLP_W3 && p < RDP_MLP_B3) bound = 0.3015f; // sqrt(6 / 66)
		const float w = u * bound;
		s.w32[p] = w;
		s.w16[p] = __float2half_rn(w);
		s.adam_m[p] = 0.0f;
		s.adam_v[p] = 0.0f;
		s.grad[p] = 0.0f;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) *s.adam_t = 0u;
}

constexpr size_t kGradSmem = sizeof(GradS);

} // namespace rdpsched

extern "C" cudaError_t rdp_sched_launch_order(const RdpSchedDev *s, const uint32_t *offsets, const uint32_t *ctrl,
                                              const uint32_t *nonempty, uint32_t blocks, cudaStream_t stream)
{
	using namespace rdpsched;
	k_tile_predict<<<blocks, WARPS * 32, 0, stream>>>(*s, offsets, ctrl, nonempty);
	k_bucket_scan<<<1, RDP_SCHED_BUCKETS, 0, stream>>>(*s, ctrl);
	k_bucket_scatter<<<blocks, 256, 0, stream>>>(*s, ctrl, nonempty);
	return cudaGetLastError();
}

static cudaError_t ensure_grad_smem()
{
	static bool done = false;
	if (done) return cudaSuccess;
	cudaError_t e = cudaFuncSetAttribute(rdpsched::k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                     int(rdpsched::kGradSmem));
	if (e == cudaSuccess) done = true;
	return e;
}

extern "C" cudaError_t rdp_sched_launch_train(const RdpSchedDev *s, const uint32_t *ctrl, const uint32_t *nonempty,
                                              const uint32_t *cycles, uint32_t blocks, cudaStream_t stream)
{
	using namespace rdpsched;
	cudaError_t e = ensure_grad_smem();
	if (e != cudaSuccess) return e;
	k_loss_clear<<<1, 1, 0, stream>>>(s->loss);
	k_mlp_grad<<<blocks, WARPS * 32, kGradSmem, stream>>>(s->w16, s->features, nullptr, 0, ctrl, nonempty, cycles,
	                                                       s->train_stride ? s->train_stride : 1u, s->grad, s->loss);
	k_mlp_adam<<<1, 1024, 0, stream>>>(*s);
	return cudaGetLastError();
}

extern "C" cudaError_t rdp_sched_launch_grad(const __half *w16, const float *features, const float *targets, uint32_t n,
                                             float *grads, float *loss, cudaStream_t stream)
{
	using namespace rdpsched;
	cudaError_t e = ensure_grad_smem();
	if (e != cudaSuccess) return e;
	uint32_t blocks = (n + WARPS - 1) / WARPS;
	if (blocks > 256) blocks = 256;
	if (!blocks) blocks = 1;
	k_mlp_grad<<<blocks, WARPS * 32, kGradSmem, stream>>>(w16, features, targets, n, nullptr, nullptr, nullptr, 1u, grads,
	                                                       loss);
	return cudaGetLastError();
}

extern "C" cudaError_t rdp_sched_launch_forward(const __half *w16, const float *features, uint32_t n, float *out,
                                                cudaStream_t stream)
{
	using namespace rdpsched;
	uint32_t blocks = (n + WARPS - 1) / WARPS;
	if (blocks > 1024) blocks = 1024;
	if (!blocks) blocks = 1;
	k_mlp_forward<<<blocks, WARPS * 32, 0, stream>>>(w16, features, n, out);
	return cudaGetLastError();
}

extern "C" cudaError_t rdp_sched_init_weights(const RdpSchedDev *s, uint32_t seed, cudaStream_t stream)
{
	rdpsched::k_mlp_init<<<8, 1024, 0, stream>>>(*s, seed);
	return cudaGetLastError();
}
