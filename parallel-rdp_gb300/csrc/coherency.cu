/*
 * RDRAM coherency between the caller's RDRAM (host memory, registered and mapped into the device's
 * address space) and the device copy the rasteriser works on -- the reference's incoherent-host
 * path (rdp_renderer.cpp:2523-2907, shaders/masked_rdram_resolve.comp, rdp_device.cpp:1195-1258).
 *
 * The GPU keeps a write mask of one bit per RDRAM byte: the pixel stores set the bits of the bytes
 * they write.  Two kernels move whole pages under that mask, reading or writing the caller's host
 * memory directly over the chip-to-chip link (no staging copy):
 *   k_coh_in  -- before a pass reads a page: the host's bytes replace the device's, except bytes the
 *                GPU has written and not yet returned to the host (those stay: GPU writes win, as in
 *                the reference's masked copy);
 *   k_coh_out -- when a timeline value is signalled: the bytes the GPU wrote go to the host, the
 *                others are left alone (the reference's masked read-back), and the mask is cleared.
 * One CTA per page, one thread per 32 bytes (one mask word).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "rdp_types.h"
#include "rdp_coherency.h"

namespace {

constexpr int kThreads = RDP_RDRAM_PAGE_BYTES / 32;

// Byte mask (0xff per selected byte) of the 4 bytes of word k of a 32-byte line from its mask bits.
__device__ __forceinline__ uint32_t byte_mask(uint32_t m, int k)
{
	const uint32_t b = (m >> (4 * k)) & 15u;
	return ((b & 1u) ? 0x000000ffu : 0u) | ((b & 2u) ? 0x0000ff00u : 0u) | ((b & 4u) ? 0x00ff0000u : 0u) |
	       ((b & 8u) ? 0xff000000u : 0u);
}

__device__ __forceinline__ void locate(const RdpCohList &L, uint32_t &inst, size_t &off)
{
	const uint32_t e = L.entry[blockIdx.x];
	inst = e >> 24;
	off = size_t(e & 0xffffffu) * RDP_RDRAM_PAGE_BYTES + threadIdx.x * 32u;
}

__global__ void __launch_bounds__(kThreads) k_coh_in(const RdpCohList L)
{
	uint32_t inst;
	size_t off;
	locate(L, inst, off);
	const uint32_t m = L.wmask[inst][off >> 5];
	if (m == 0xffffffffu) return; // every byte of the line is the GPU's
	const uint8_t *h = L.host[inst] + off;
	uint8_t *d = L.dev[inst] + off;
	if ((L.host_aligned >> inst) & 1u)
	{
		// Host bytes: fetched again on every access (__ldcv), never from a cached line.
		uint4 hv[2] = { __ldcv(reinterpret_cast<const uint4 *>(h)), __ldcv(reinterpret_cast<const uint4 *>(h + 16)) };
		if (m)
		{
			const uint4 *dv = reinterpret_cast<const uint4 *>(d);
			uint4 cur[2] = { dv[0], dv[1] };
			uint32_t *hw = reinterpret_cast<uint32_t *>(hv);
			const uint32_t *cw = reinterpret_cast<const uint32_t *>(cur);
#pragma unroll
			for (int k = 0; k < 8; k++)
			{
				const uint32_t bm = byte_mask(m, k);
				hw[k] = (cw[k] & bm) | (hw[k] & ~bm);
			}
		}
		reinterpret_cast<uint4 *>(d)[0] = hv[0];
		reinterpret_cast<uint4 *>(d)[1] = hv[1];
	}
	else
	{
		for (int b = 0; b < 32; b++)
			if (!((m >> b) & 1u)) d[b] = __ldcv(reinterpret_cast<const unsigned char *>(h) + b);
	}
}

__global__ void __launch_bounds__(kThreads) k_coh_out(const RdpCohList L)
{
	uint32_t inst;
	size_t off;
	locate(L, inst, off);
	uint32_t *mw = L.wmask[inst] + (off >> 5);
	const uint32_t m = *mw;
	if (!m) return;
	const uint8_t *d = L.dev[inst] + off;
	uint8_t *h = L.host[inst] + off;
	if (m == 0xffffffffu && ((L.host_aligned >> inst) & 1u))
	{
		// Host bytes: written through to the caller's memory (__stwt).
		__stwt(reinterpret_cast<uint4 *>(h), reinterpret_cast<const uint4 *>(d)[0]);
		__stwt(reinterpret_cast<uint4 *>(h) + 1, reinterpret_cast<const uint4 *>(d)[1]);
	}
	else
	{
		const uint32_t *dw = reinterpret_cast<const uint32_t *>(d);
		for (int k = 0; k < 8; k++)
		{
			const uint32_t nib = (m >> (4 * k)) & 15u;
			if (nib == 15u && ((L.host_aligned >> inst) & 1u))
				__stwt(reinterpret_cast<unsigned int *>(h) + k, dw[k]);
			else
				for (int b = 0; b < 4; b++)
					if ((nib >> b) & 1u) __stwt(reinterpret_cast<unsigned char *>(h) + 4 * k + b, d[4 * k + b]);
		}
	}
	*mw = 0u;
}

} // namespace

extern "C" cudaError_t rdp_coherency_launch(const RdpCohList *list, int to_host, cudaStream_t stream)
{
	if (!list->count) return cudaSuccess;
	if (to_host)
		k_coh_out<<<list->count, kThreads, 0, stream>>>(*list);
	else
		k_coh_in<<<list->count, kThreads, 0, stream>>>(*list);
	return cudaGetLastError();
}
