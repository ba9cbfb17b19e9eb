// lexgb_cnn.cuh - common includes of the learned SGS correction's CNN kernels.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/lexgb.h"

namespace lexgb {
// tcgen05 convolution (kernels_cnn_tc.cu): shape rule, launch, one-time set-up, timeout count
bool conv_tc_fits(int nx, int ny, int nz, int cin, int cout, const void* x, const void* pre, const void* ybf,
                  const void* yf);
cudaError_t launch_conv_tc(int nx, int ny, int nz, int cin, int cout, const void* x, const void* w, const float* bias,
                           float* pre, void* ybf, float* yf, int gelu, int creal, cudaStream_t st, bool pdl);
cudaError_t conv_tc_prepare();
cudaError_t conv_tc_take_timeouts(unsigned int* n);
// tcgen05 weight gradient (kernels_cnn_tc.cu): dw[27][cout][cin] += sum_p g[p][co] x[p+off][ci]
bool conv_dw_tc_fits(int nx, int ny, int nz, int cin, int cout, int gstride, const void* x, const void* g,
                     const float* dw);
cudaError_t launch_conv_dw_tc(int nx, int ny, int nz, int cin, int cout, int gstride, const void* x, const void* g,
                              float* dw, cudaStream_t st);
}  // namespace lexgb
