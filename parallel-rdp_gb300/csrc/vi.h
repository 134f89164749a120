/* Video Interface (scanout) kernels: see vi.cu. */
#ifndef RDP_VI_H
#define RDP_VI_H
#include <stdint.h>
#endif
