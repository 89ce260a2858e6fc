/* cfgs_plain.h — the plain GPU path of the rasteriser: the published 3D Gaussian
 * Splatting rasteriser's structure (Kerbl et al. 2023, the CUDA rasteriser that
 * CF-3DGS's submodules/diff-gaussian-rasterization builds), written for this library
 * as the GPU comparison point for its tuned kernels. The upstream CUDA source is not
 * part of the CF-3DGS tree, so it cannot be built and timed beside them.
 *
 * What follows the published structure here:
 *  - binning: an inclusive scan of the tiles touched per Gaussian (read back to the
 *    host to size the instance buffers), one thread per Gaussian writing its 64-bit
 *    keys (tile << 32 | depth bits) and Gaussian ids, one radix sort of the keys over
 *    32 + bits(tiles) bits (CUB DeviceRadixSort), and per-tile ranges found at the key
 *    boundaries of the sorted list;
 *  - forward: one 256-thread block per 16x16 tile and one thread per pixel; rounds of
 *    256 instances fetched into shared memory by the block, every pixel testing every
 *    instance until the whole block is saturated; colour and depth read from global
 *    memory for each contribution;
 *  - backward: the same block and pixel mapping walked back to front, each
 *    (pixel, Gaussian) contribution adding its gradient terms to the Gaussian's
 *    accumulators with global atomic adds, then the per-Gaussian backward.
 * The preprocess (cfgs_preprocess_forward) and the per-Gaussian backward kernel are the
 * library's own: both are one thread per Gaussian in the published structure too.
 * The per-pixel arithmetic is the library's (same operation order and exponential), so
 * the plain forward's images, contributor counts and transmittances equal the tuned
 * path's bit for bit; the backward's atomic sums differ from run to run by rounding.
 *
 * Same conventions as cfgs.h: int status, caller-owned device buffers, a stream. */
#ifndef CFGS_PLAIN_H_
#define CFGS_PLAIN_H_

#include "cfgs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Bytes of the plain path's workspace for N Gaussians, up to `capacity` tile instances,
 * on a width x height image: offsets, key/id buffers, tile ranges, per-Gaussian gradient
 * accumulators and the sort's temporary storage. 0 when the sort's storage query fails. */
size_t cfgs_plain_work_bytes(int32_t num_gaussians, int64_t capacity, int32_t width, int32_t height);

/* Binning after cfgs_preprocess_forward (geom holds the tiles touched, rectangles and
 * depths): scan, blocking read of the instance count into *num_rendered, keys, sort,
 * ranges. CFGS_ERR_CAPACITY (with *num_rendered set) when the count exceeds `capacity`:
 * grow the workspace and call again. */
int cfgs_plain_bin(const CfgsSettings* settings, int32_t num_gaussians, const void* geom, void* work,
                   int64_t capacity, int64_t* num_rendered, void* stream);

/* Per-pixel compositing over the ranges of cfgs_plain_bin. Writes colour [3,H,W], depth
 * [1,H,W] and alpha [1,H,W] (depth and alpha may be NULL) and the final transmittance
 * and contributor count of each pixel into the image workspace for the backward. */
int cfgs_plain_render_forward(const CfgsSettings* settings, int32_t num_gaussians, const void* geom, void* image,
                              const void* work, int64_t capacity, float* out_color, float* out_depth,
                              float* out_alpha, void* stream);

/* The backward of one cfgs_plain_render_forward: per-pixel atomic accumulation, then
 * the per-Gaussian chain into the eight gradient arrays of `grads` (as cfgs_backward). */
int cfgs_plain_backward(const CfgsSettings* settings, const CfgsGaussians* gaussians, const int32_t* radii,
                        const void* geom, const void* image, void* work, int64_t capacity, const float* dL_dcolor,
                        const float* dL_ddepth, const float* dL_dalpha, const CfgsGradients* grads, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CFGS_PLAIN_H_ */
