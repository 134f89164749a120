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
 * One CTA per page; thread t moves bytes 16t .. 16t+15 of each 2 KiB half of the page, so that one
 * warp instruction covers 512 contiguous bytes of the link (whole 32-byte sectors, each read or
 * written once).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "rdp_types.h"
#include "rdp_coherency.h"

namespace {

constexpr int kThreads = 128;
constexpr uint32_t kHalf = kThreads * 16; // bytes of a page one CTA instruction covers
static_assert(RDP_RDRAM_PAGE_BYTES == 2 * kHalf, "two 16-byte pieces per thread and page");

// Byte mask (0xff per selected byte) of the 4 bytes of word k of a 16-byte piece from its mask bits.
__device__ __forceinline__ uint32_t byte_mask(uint32_t m, int k)
{
	const uint32_t b = (m >> (4 * k)) & 15u;
	return ((b & 1u) ? 0x000000ffu : 0u) | ((b & 2u) ? 0x0000ff00u : 0u) | ((b & 4u) ? 0x00ff0000u : 0u) |
	       ((b & 8u) ? 0xff000000u : 0u);
}

// Instance slot and byte offset of this CTA's page.
__device__ __forceinline__ void locate(const RdpCohList &L, uint32_t &inst, size_t &page)
{
	const uint32_t e = L.entry[blockIdx.x];
	inst = e >> 24;
	page = size_t(e & 0xffffffu) * RDP_RDRAM_PAGE_BYTES;
}

// The 16 mask bits of the piece at byte offset `off` (a multiple of 16).
__device__ __forceinline__ uint32_t piece_mask(const uint32_t *wmask, size_t off)
{
	return (wmask[off >> 5] >> (off & 16u)) & 0xffffu;
}

__global__ void __launch_bounds__(kThreads) k_coh_in(const RdpCohList L)
{
	uint32_t inst;
	size_t page;
	locate(L, inst, page);
	const bool aligned = (L.host_aligned >> inst) & 1u;
#pragma unroll
	for (int half = 0; half < 2; half++)
	{
		const size_t off = page + half * kHalf + threadIdx.x * 16u;
		const uint32_t m = piece_mask(L.wmask[inst], off);
		if (m == 0xffffu) continue; // every byte of the piece is the GPU's
		const uint8_t *h = L.host[inst] + off;
		uint8_t *d = L.dev[inst] + off;
		if (aligned)
		{
			// Host bytes: fetched again on every access (__ldcv), never from a cached line.
			uint4 hv = __ldcv(reinterpret_cast<const uint4 *>(h));
			if (m)
			{
				const uint4 cur = *reinterpret_cast<const uint4 *>(d);
				hv.x = (cur.x & byte_mask(m, 0)) | (hv.x & ~byte_mask(m, 0));
				hv.y = (cur.y & byte_mask(m, 1)) | (hv.y & ~byte_mask(m, 1));
				hv.z = (cur.z & byte_mask(m, 2)) | (hv.z & ~byte_mask(m, 2));
				hv.w = (cur.w & byte_mask(m, 3)) | (hv.w & ~byte_mask(m, 3));
			}
			*reinterpret_cast<uint4 *>(d) = hv;
		}
		else
		{
			for (int b = 0; b < 16; b++)
				if (!((m >> b) & 1u)) d[b] = __ldcv(reinterpret_cast<const unsigned char *>(h) + b);
		}
	}
}

__global__ void __launch_bounds__(kThreads) k_coh_out(const RdpCohList L)
{
	uint32_t inst;
	size_t page;
	locate(L, inst, page);
	const bool aligned = (L.host_aligned >> inst) & 1u;
	uint32_t *wmask = L.wmask[inst];
	// Both pieces' masks and device bytes are loaded before any is written out.
	size_t off[2];
	uint32_t m[2];
	uint4 v[2];
#pragma unroll
	for (int half = 0; half < 2; half++)
	{
		off[half] = page + half * kHalf + threadIdx.x * 16u;
		m[half] = piece_mask(wmask, off[half]);
		v[half] = *reinterpret_cast<const uint4 *>(L.dev[inst] + off[half]);
	}
#pragma unroll
	for (int half = 0; half < 2; half++)
	{
		uint8_t *h = L.host[inst] + off[half];
		if (m[half] == 0xffffu && aligned)
		{
			// Host bytes: written through to the caller's memory (__stwt).
			__stwt(reinterpret_cast<uint4 *>(h), v[half]);
		}
		else if (m[half])
		{
			const uint32_t dw[4] = { v[half].x, v[half].y, v[half].z, v[half].w };
			for (int k = 0; k < 4; k++)
			{
				const uint32_t nib = (m[half] >> (4 * k)) & 15u;
				if (nib == 15u && aligned)
					__stwt(reinterpret_cast<unsigned int *>(h) + k, dw[k]);
				else
					for (int b = 0; b < 4; b++)
						if ((nib >> b) & 1u) __stwt(h + 4 * k + b, uint8_t(dw[k] >> (8 * b)));
			}
		}
		// The mask word covers this piece and its neighbour's (thread t ^ 1, same warp): both have
		// read it before the even thread clears it.
		const uint32_t pair = m[half] | __shfl_xor_sync(0xffffffffu, m[half], 1);
		if (!(threadIdx.x & 1u) && pair) wmask[off[half] >> 5] = 0u;
	}
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
