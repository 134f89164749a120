/*
 * Internal upscaling of the GB300 RDP path (the reference's render_pass_upscaled and
 * update_upscaled_domain_{pre,post,resolve}.comp): the kernels that keep the multisampled copy of
 * RDRAM in step with RDRAM and resolve it for super-sampled readback (upscale.cu).
 */
#ifndef RDP_UPSCALE_H
#define RDP_UPSCALE_H

#include <cuda_runtime.h>
#include <stdint.h>

typedef struct RdpUpscaleDomain
{
	uint8_t *rdram, *hidden;      /* native RDRAM / hidden RDRAM (device) */
	uint8_t *reference;           /* what the multisampled copy reflects of RDRAM (rdram_size bytes) */
	uint8_t *ms_rdram, *ms_hidden; /* samples^2 slices of rdram_size / rdram_size / 2 bytes */
	uint32_t *ssaa_mask;          /* super-sampled write mask (after the RDRAM slices), or null */
	uint32_t *wmask;              /* coherency write mask of RDRAM (1 bit per byte), or null */
	uint32_t rdram_size, hidden_size;
	uint32_t samples;             /* factor^2 */
} RdpUpscaleDomain;

#ifdef __cplusplus
extern "C" {
#endif
/* update_upscaled_domain_pre.comp (post = 0) / update_upscaled_domain_post.comp (post = 1) over
 * `pixels` elements of 2^psl2 bytes from addr (word aligned, rounded up to whole words) and, unless
 * depth_addr equals addr, as many 16-bit elements from depth_addr. */
cudaError_t rdp_upscale_sync(const RdpUpscaleDomain *d, uint32_t addr, uint32_t depth_addr, uint32_t pixels,
                             uint32_t psl2, int post, cudaStream_t stream);
/* clear_super_sampled_write_mask.comp over the 4x4 blocks of a width x height image. */
cudaError_t rdp_ssaa_clear_mask(const RdpUpscaleDomain *d, uint32_t width, uint32_t height, cudaStream_t stream);
/* update_upscaled_domain_resolve.comp for the image (addr, depth_addr, width x height, psl2). */
cudaError_t rdp_ssaa_resolve(const RdpUpscaleDomain *d, uint32_t addr, uint32_t depth_addr, uint32_t width,
                             uint32_t height, uint32_t psl2, int dither, cudaStream_t stream);
#ifdef __cplusplus
}
#endif
#endif
