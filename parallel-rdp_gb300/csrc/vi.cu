/* Video Interface scanout (filled in by the VI stage). */
#include <cuda_runtime.h>
#include "../../include/rdp_cuda.h"
#include "vi.h"

extern "C" int rdp_cp_scanout_sync(rdp_cp *cp, const rdp_scanout_options *opts, uint32_t *rgba_out, uint32_t *width,
                                   uint32_t *height)
{
	(void)cp; (void)opts; (void)rgba_out;
	if (width) *width = 0;
	if (height) *height = 0;
	return RDP_ERR_UNSUPPORTED;
}
