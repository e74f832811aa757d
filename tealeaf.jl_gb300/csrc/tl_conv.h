// tl_conv.h -- host entry points of the warm-start network kernels used
// inside the library (the C ABI adds the training entry points).
#pragma once

#include <cuda_runtime.h>

#include "../../include/tealeaf_gb300.h"

int tl_conv_forward(const void *x, const void *w, const float *bias, const void *gz, void *z, void *out, float *out32,
                    int N, int H, int W, int cin, int cout, int mode, cudaStream_t st);
int tl_warm_features_launch(const tl_warm_crop *crops, int B, int H, int W, void *feat, cudaStream_t st);

// Layer shapes of the network (input channels padded to 16, output to 16).
constexpr int TL_WARM_LAYERS = 6;
constexpr int TL_WARM_CIN[TL_WARM_LAYERS] = {16, 32, 32, 32, 32, 32};
constexpr int TL_WARM_COUT[TL_WARM_LAYERS] = {32, 32, 32, 32, 32, 16};
