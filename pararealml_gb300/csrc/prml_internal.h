/* Internal helpers shared by the translation units of libprml_gb300.so. */
#ifndef PRML_INTERNAL_H
#define PRML_INTERNAL_H

#include <cuda.h>

#include <string>

#include "pararealml_gb300.h"

/* Records `msg` as the calling thread's last error and returns `code`. */
int prml_set_error(int code, const std::string& msg);

/* The calling thread's current CUDA context (driver handle), or NULL. */
void* prml_current_context();

/* Encodes a tiled TMA map (no interleave, zero fill outside the tensor,
 * swizzle_bytes 0 / 32 / 64 / 128) through the driver loaded by the
 * runtime; dims/box innermost first, strides in bytes for dims 1..rank-1. */
extern "C" int prml_tensor_map_tiled(CUtensorMap* map, CUtensorMapDataType dtype, unsigned rank,
                                     const void* base, const unsigned long long* dims,
                                     const unsigned long long* strides, const unsigned* box,
                                     int swizzle_bytes);

/* The tcgen05 32 -> 32 convolution (prml_cnn_tc.cu): mode 0 forward with
 * bias + ReLU, mode 1 data gradient with the ReLU mask. */
int prml_cnn_tc_enabled();
int prml_cnn_mid_conv_tc(int mode, const void* x, const void* w, const float* bias, const void* mask, void* y,
                         int B, int H, int W, void* stream);
/* The tcgen05 weight gradient of a 32 -> 32 convolution: per-CTA partial
 * sums [tap][co][ci] into `partial` (at most `parts` CTAs; *used = the
 * number launched). */
int prml_cnn_mid_wgrad_tc(const void* x, const void* g, float* partial, int parts, int* used, int B, int H, int W,
                          void* stream);

#endif
