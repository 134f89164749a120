/* Launch interface of the RDRAM coherency kernels (coherency.cu). */
#ifndef RDP_COHERENCY_H
#define RDP_COHERENCY_H

#include <cuda_runtime.h>
#include <stdint.h>

/* Instances and pages per launch: the list travels as the kernel's parameter block (which holds
 * up to 32,764 bytes), so no device buffer is needed for it. */
#define RDP_COH_MAX_INSTANCES 16
#define RDP_COH_MAX_PAGES 7168

/* Pages of up to RDP_COH_MAX_INSTANCES instances: entry = instance slot << 24 | page index. */
typedef struct RdpCohList
{
	uint8_t *host[RDP_COH_MAX_INSTANCES];   /* mapped host RDRAM bases */
	uint8_t *dev[RDP_COH_MAX_INSTANCES];    /* device RDRAM bases */
	uint32_t *wmask[RDP_COH_MAX_INSTANCES]; /* device write masks (1 bit per byte) */
	uint32_t host_aligned;                  /* bit i: host[i] is 16-byte aligned */
	uint32_t count;
	uint32_t entry[RDP_COH_MAX_PAGES];
} RdpCohList;

#ifdef __cplusplus
extern "C" {
#endif
/* to_host = 0: masked host -> device merge of the listed pages (k_coh_in); 1: masked device -> host
 * write-back, clearing the mask (k_coh_out). */
cudaError_t rdp_coherency_launch(const RdpCohList *list, int to_host, cudaStream_t stream);
#ifdef __cplusplus
}
#endif
#endif
