/*
 * Upscaled-domain kernels for sm_103a (the reference's update_upscaled_domain_pre.comp,
 * update_upscaled_domain_post.comp, clear_super_sampled_write_mask.comp and
 * update_upscaled_domain_resolve.comp; dispatched by Renderer::submit_update_upscaled_domain,
 * rdp_renderer.cpp:1937-2085).
 *
 * The multisampled copy holds samples = factor^2 slices of RDRAM and of hidden RDRAM; the
 * reference copy holds the RDRAM bytes the multisampled copy already reflects.
 *   k_upscale_sync (pre)  -- each element of RDRAM that differs from the reference copy is written
 *                            to every slice with its hidden bits, and recorded in the reference;
 *   k_upscale_sync (post) -- the reference copy takes RDRAM (after a 1x pass that the upscaled
 *                            pass renders again);
 *   k_ssaa_resolve        -- every native pixel a sample wrote takes the mean of its samples
 *                            (colour) or its first sample (depth), in RDRAM and the reference.
 * One thread per element / pixel; everything is byte addressed little-endian like RDRAM.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "rdp_upscale.h"

namespace {

constexpr int kThreads = 256;
__constant__ uint8_t kBayer[16] = { 0, 4, 1, 5, 4, 0, 5, 1, 3, 7, 2, 6, 7, 3, 6, 2 };

__device__ __forceinline__ uint32_t load_n(const uint8_t *p, uint32_t bytes)
{
	if (bytes == 1) return p[0];
	if (bytes == 2) return *reinterpret_cast<const uint16_t *>(p);
	return *reinterpret_cast<const uint32_t *>(p);
}
__device__ __forceinline__ void store_n(uint8_t *p, uint32_t bytes, uint32_t v)
{
	if (bytes == 1) p[0] = uint8_t(v);
	else if (bytes == 2) *reinterpret_cast<uint16_t *>(p) = uint16_t(v);
	else *reinterpret_cast<uint32_t *>(p) = v;
}

__device__ void sync_element(const RdpUpscaleDomain &d, uint32_t index, uint32_t psl2, bool post)
{
	index &= (d.rdram_size >> psl2) - 1;
	const uint32_t bytes = 1u << psl2, b = index << psl2, hs = d.rdram_size >> 1;
	const uint32_t real = load_n(d.rdram + b, bytes);
	if (post)
	{
		store_n(d.reference + b, bytes, real);
		return;
	}
	if (real == load_n(d.reference + b, bytes)) return;
	for (uint32_t i = 0; i < d.samples; i++)
	{
		store_n(d.ms_rdram + size_t(i) * d.rdram_size + b, bytes, real);
		uint8_t *mh = d.ms_hidden + size_t(i) * hs;
		if (psl2 == 0)
		{
			const uint32_t m = index ^ 3u;
			if (m & 1u) mh[m >> 1] = d.hidden[(m >> 1) & (d.hidden_size - 1)];
		}
		else if (psl2 == 1)
		{
			const uint32_t m = index ^ 1u;
			mh[m] = d.hidden[m & (d.hidden_size - 1)];
		}
		else
		{
			mh[2 * index] = d.hidden[(2 * index) & (d.hidden_size - 1)];
			mh[2 * index + 1] = d.hidden[(2 * index + 1) & (d.hidden_size - 1)];
		}
	}
	store_n(d.reference + b, bytes, real);
}

__global__ void __launch_bounds__(kThreads) k_upscale_sync(const RdpUpscaleDomain d, uint32_t color_base,
                                                           uint32_t depth_base, uint32_t pixels, uint32_t psl2,
                                                           int alias, int post)
{
	const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
	if (i >= pixels) return;
	sync_element(d, color_base + i, psl2, post != 0);
	if (!alias) sync_element(d, depth_base + i, 1, post != 0);
}

__global__ void __launch_bounds__(kThreads) k_ssaa_clear(uint32_t *mask, uint32_t words)
{
	const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
	if (i < words) mask[i] = 0u;
}

// Marks `bytes` bytes of RDRAM from byte b as written by the GPU (the coherency write mask).
__device__ __forceinline__ void mark_rdram(const RdpUpscaleDomain &d, uint32_t b, uint32_t bytes)
{
	if (!d.wmask) return;
	atomicOr(d.wmask + (b >> 5), ((1u << bytes) - 1u) << (b & 31u));
}

__global__ void __launch_bounds__(kThreads) k_ssaa_resolve(const RdpUpscaleDomain d, uint32_t color_base,
                                                           uint32_t depth_base, uint32_t width, uint32_t height,
                                                           uint32_t psl2, int alias, int dither)
{
	const uint32_t x = blockIdx.x * kThreads + threadIdx.x, y = blockIdx.y;
	if (x >= width || y >= height) return;
	const uint32_t n = d.samples;
	const uint32_t index = y * width + x;
	const uint32_t wm = d.ssaa_mask[(x >> 2) + (y >> 2) * ((width + 3) >> 2)] >> (2 * ((x & 3) + 4 * (y & 3)));
	if (wm & 1u)
	{
		uint32_t ci = color_base + index;
		if (psl2 == 0)
		{
			// The reference sums the first sample `samples` times: the result is that sample.
			ci = (ci & (d.rdram_size - 1)) ^ 3u;
			const uint8_t v = d.ms_rdram[ci];
			d.rdram[ci] = v;
			d.reference[ci] = v;
			mark_rdram(d, ci, 1);
		}
		else if (psl2 == 1)
		{
			ci = (ci & ((d.rdram_size >> 1) - 1)) ^ 1u;
			uint32_t r = 0, g = 0, b = 0, a = 0;
			for (uint32_t i = 0; i < n; i++)
			{
				const uint32_t v = reinterpret_cast<const uint16_t *>(d.ms_rdram + size_t(i) * d.rdram_size)[ci];
				r += (v >> 11) & 0x1fu;
				g += (v >> 6) & 0x1fu;
				b += (v >> 1) & 0x1fu;
				a += v & 1u;
			}
			if (dither)
			{
				// 4x4 ordered dither of the mean (update_upscaled_domain_resolve.comp:115-142).
				const uint32_t dv = kBayer[(y & 3u) * 4u + (x & 3u)] * n;
				r = (8 * r + dv) / (8 * n);
				g = (8 * g + dv) / (8 * n);
				b = (8 * b + dv) / (8 * n);
				a = (8 * a + dv) / (8 * n);
			}
			else
			{
				r = (r + (n >> 1)) / n;
				g = (g + (n >> 1)) / n;
				b = (b + (n >> 1)) / n;
				a = (a + (n >> 1)) / n;
			}
			const uint16_t enc = uint16_t((r << 11) | (g << 6) | (b << 1) | a);
			reinterpret_cast<uint16_t *>(d.rdram)[ci] = enc;
			reinterpret_cast<uint16_t *>(d.reference)[ci] = enc;
			mark_rdram(d, ci * 2, 2);
		}
		else
		{
			ci &= (d.rdram_size >> 2) - 1;
			uint32_t sum[4] = { 0, 0, 0, 0 };
			for (uint32_t i = 0; i < n; i++)
			{
				const uint32_t v = reinterpret_cast<const uint32_t *>(d.ms_rdram + size_t(i) * d.rdram_size)[ci];
#pragma unroll
				for (int c = 0; c < 4; c++) sum[c] += (v >> (24 - 8 * c)) & 0xffu;
			}
			uint32_t enc = 0;
#pragma unroll
			for (int c = 0; c < 4; c++) enc |= (((sum[c] + (n >> 1)) / n) & 0xffu) << (24 - 8 * c);
			reinterpret_cast<uint32_t *>(d.rdram)[ci] = enc;
			reinterpret_cast<uint32_t *>(d.reference)[ci] = enc;
			mark_rdram(d, ci * 4, 4);
		}
	}
	if (!alias && (wm & 2u))
	{
		// Depth: the first sample (it lines up with the native pixel).
		const uint32_t di = ((depth_base + index) & ((d.rdram_size >> 1) - 1)) ^ 1u;
		const uint16_t v = reinterpret_cast<const uint16_t *>(d.ms_rdram)[di];
		reinterpret_cast<uint16_t *>(d.rdram)[di] = v;
		reinterpret_cast<uint16_t *>(d.reference)[di] = v;
		mark_rdram(d, di * 2, 2);
	}
}

} // namespace

extern "C" cudaError_t rdp_upscale_sync(const RdpUpscaleDomain *d, uint32_t addr, uint32_t depth_addr, uint32_t pixels,
                                        uint32_t psl2, int post, cudaStream_t stream)
{
	addr &= ~3u;
	depth_addr &= ~3u;
	const uint32_t align = 4u >> psl2;
	pixels = (pixels + align - 1) & ~(align - 1);
	if (!pixels) return cudaSuccess;
	k_upscale_sync<<<(pixels + kThreads - 1) / kThreads, kThreads, 0, stream>>>(
		*d, addr >> psl2, depth_addr >> 1, pixels, psl2, addr == depth_addr, post);
	return cudaGetLastError();
}

extern "C" cudaError_t rdp_ssaa_clear_mask(const RdpUpscaleDomain *d, uint32_t width, uint32_t height, cudaStream_t stream)
{
	const uint32_t words = ((width + 3) / 4) * ((height + 3) / 4);
	if (!words || !d->ssaa_mask) return cudaSuccess;
	k_ssaa_clear<<<(words + kThreads - 1) / kThreads, kThreads, 0, stream>>>(d->ssaa_mask, words);
	return cudaGetLastError();
}

extern "C" cudaError_t rdp_ssaa_resolve(const RdpUpscaleDomain *d, uint32_t addr, uint32_t depth_addr, uint32_t width,
                                        uint32_t height, uint32_t psl2, int dither, cudaStream_t stream)
{
	if (!width || !height || !d->ssaa_mask) return cudaSuccess;
	k_ssaa_resolve<<<dim3((width + kThreads - 1) / kThreads, height), kThreads, 0, stream>>>(
		*d, addr >> psl2, depth_addr >> 1, width, height, psl2, addr == depth_addr, dither);
	return cudaGetLastError();
}
