/* Launch interface of the RDP kernels (rdp_kernels.cu). */
#ifndef RDP_KERNELS_H
#define RDP_KERNELS_H

#include <cuda_runtime.h>
#include "rdp_types.h"

typedef struct RdpLaunch
{
	const RdpPrimIn *prims_in;
	uint32_t num_prims;
	const uint32_t *words;
	const uint32_t *state_blocks;
	const RdpPass *passes;
	uint32_t num_passes;
	RdpPrimGeom *geom;
	RdpPrimAttr *attr;
	RdpPrimShade *shade;
	const RdpTile *tilesets;
	const uint32_t *tmem_pass_list;
	uint32_t num_tmem_passes;
	const RdpUpload *uploads;
	uint32_t num_tile_items;
	unsigned long long *fragments;
} RdpLaunch;

#ifdef __cplusplus
extern "C" {
#endif
cudaError_t rdp_kernels_init_luts(const uint8_t *blender_lut);
cudaError_t rdp_kernels_launch(const RdpLaunch *launch, cudaStream_t stream);
#ifdef __cplusplus
}
#endif
#endif
