/*
 * Learned tile scheduling of the GB300 RDP path.
 *
 * A small MLP (16 -> 64 -> 64 -> 1, ReLU, FP16 weights, FP32 accumulation) predicts the
 * blend cost of every non-empty tile from binning features (its (primitive, tile) pair count
 * and the fractions of its primitives in 2-cycle / copy / fill mode, textured, perspective,
 * depth-tested, depth-written, blending, anti-aliased, alpha-tested, bilinear, plus the image
 * format).  The prediction only orders k_blend's persistent work queue longest-first; the
 * order never changes a pixel.  The network is trained on the GPU, online, on the cycles
 * k_blend measures per tile with clock64, by this file's own forward / backward kernels and an
 * Adam update.
 */
#ifndef RDP_SCHED_H
#define RDP_SCHED_H

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include "rdp_types.h"

#define RDP_MLP_IN 16
#define RDP_MLP_HIDDEN 64
/* Packed parameter layout: W1[64][16], b1[64], W2[64][64], b2[64], W3[64], b3. */
#define RDP_MLP_W1 0
#define RDP_MLP_B1 (RDP_MLP_W1 + RDP_MLP_HIDDEN * RDP_MLP_IN)
#define RDP_MLP_W2 (RDP_MLP_B1 + RDP_MLP_HIDDEN)
#define RDP_MLP_B2 (RDP_MLP_W2 + RDP_MLP_HIDDEN * RDP_MLP_HIDDEN)
#define RDP_MLP_W3 (RDP_MLP_B2 + RDP_MLP_HIDDEN)
#define RDP_MLP_B3 (RDP_MLP_W3 + RDP_MLP_HIDDEN)
#ifndef RDP_MLP_PARAMS /* also defined by the public header rdp_cuda.h */
#define RDP_MLP_PARAMS (RDP_MLP_B3 + 1)
#endif
static_assert(RDP_MLP_PARAMS == RDP_MLP_B3 + 1, "packed MLP parameter count");
#define RDP_SCHED_BUCKETS 1024

/* Per-primitive feature bits (k_prim_setup) that the tile features count (k_expand). */
enum
{
	RDP_FEAT_MULTI_CYCLE = 0, RDP_FEAT_COPY, RDP_FEAT_FILL, RDP_FEAT_TEXEL0, RDP_FEAT_TEXEL1, RDP_FEAT_PERSPECTIVE,
	RDP_FEAT_DEPTH_TEST, RDP_FEAT_DEPTH_UPDATE, RDP_FEAT_BLEND, RDP_FEAT_AA, RDP_FEAT_ALPHA_TEST, RDP_FEAT_BILERP,
	RDP_FEAT_NOISE, RDP_FEAT_COUNT
};
/* Tiles with fewer pairs than this are not evaluated: they go to the end of the queue.  Order
 * matters for the heavy tiles; on the 64-instance batched workload thresholds of 16, 64, 256 and
 * 512 pairs gave sync points of 22.30, 21.99, 21.84 and 21.84 ms (static tile order: 21.93). */
#define RDP_SCHED_MIN_PAIRS 256

#ifdef __CUDACC__
static __host__ __device__ __forceinline__ uint16_t rdp_feature_bits(uint32_t f, uint32_t d)
{
	uint32_t b = 0;
	b |= ((f & RS_MULTI_CYCLE) != 0) << RDP_FEAT_MULTI_CYCLE;
	b |= ((f & RS_COPY) != 0) << RDP_FEAT_COPY;
	b |= ((f & RS_FILL) != 0) << RDP_FEAT_FILL;
	b |= ((f & RS_USES_TEXEL0) != 0) << RDP_FEAT_TEXEL0;
	b |= ((f & RS_USES_TEXEL1) != 0) << RDP_FEAT_TEXEL1;
	b |= ((f & RS_PERSPECTIVE) != 0) << RDP_FEAT_PERSPECTIVE;
	b |= ((d & DB_DEPTH_TEST) != 0) << RDP_FEAT_DEPTH_TEST;
	b |= ((d & DB_DEPTH_UPDATE) != 0) << RDP_FEAT_DEPTH_UPDATE;
	b |= ((d & (DB_FORCE_BLEND | DB_IMAGE_READ)) != 0) << RDP_FEAT_BLEND;
	b |= (((d & DB_AA) | (f & RS_AA)) != 0) << RDP_FEAT_AA;
	b |= ((f & RS_ALPHA_TEST) != 0) << RDP_FEAT_ALPHA_TEST;
	b |= ((f & (RS_BILERP0 | RS_BILERP1)) != 0) << RDP_FEAT_BILERP;
	b |= ((f & RS_NEED_NOISE) != 0) << RDP_FEAT_NOISE;
	return uint16_t(b);
}
#endif

typedef struct RdpSchedDev
{
	__half *w16;        /* [RDP_MLP_PARAMS] weights used by inference and the training forward pass */
	float *w32;         /* [RDP_MLP_PARAMS] FP32 master weights (Adam updates these) */
	float *adam_m, *adam_v, *grad; /* [RDP_MLP_PARAMS] */
	uint32_t *adam_t;   /* Adam step counter */
	float *loss;        /* [2]: sum of squared errors and sample count of the last training step */
	uint16_t *featbits; /* [primitive capacity]: rdp_feature_bits of each primitive (k_prim_setup) */
	float *features;    /* [tile capacity][RDP_MLP_IN], indexed by tile item (k_expand) */
	float *pred;        /* [tile capacity], indexed like the non-empty tile list */
	uint32_t *bucket;   /* [tile capacity], indexed like the non-empty tile list */
	uint32_t *hist;     /* [RDP_SCHED_BUCKETS] counts; zero between launches */
	uint32_t *cursor;   /* [RDP_SCHED_BUCKETS] write positions */
	uint32_t *order;    /* [capacity]: tile items, longest predicted first */
	uint32_t capacity;
	uint32_t order_enabled, train_enabled, train_stride;
	float lr;
} RdpSchedDev;

#ifdef __cplusplus
extern "C" {
#endif
/* After k_expand (which wrote the tile features): prediction per non-empty tile, bucket sort
 * into s->order. */
cudaError_t rdp_sched_launch_order(const RdpSchedDev *s, const uint32_t *offsets, const uint32_t *ctrl,
                                   const uint32_t *nonempty, uint32_t blocks, cudaStream_t stream);
/* After k_blend: one Adam step on this launch's tiles (features, log2 of measured cycles). */
cudaError_t rdp_sched_launch_train(const RdpSchedDev *s, const uint32_t *ctrl, const uint32_t *nonempty,
                                   const uint32_t *cycles, uint32_t blocks, cudaStream_t stream);
/* Loss gradients of the packed parameters for n samples (FP16 weights, FP32 accumulation);
 * grads and loss are device buffers, zeroed by the caller.  Used by the online trainer and by
 * the gradient check against the CPU restatement. */
cudaError_t rdp_sched_launch_grad(const __half *w16, const float *features, const float *targets, uint32_t n,
                                  float *grads, float *loss, cudaStream_t stream);
/* Forward pass only: out[i] for n samples. */
cudaError_t rdp_sched_launch_forward(const __half *w16, const float *features, uint32_t n, float *out,
                                     cudaStream_t stream);
/* Fresh weights (deterministic small uniform initialisation from seed) into w32 / w16, Adam state zeroed. */
cudaError_t rdp_sched_init_weights(const RdpSchedDev *s, uint32_t seed, cudaStream_t stream);
#ifdef __cplusplus
}
#endif
#endif
