/*
 * Device rate probe: the float64 fused multiply-add rate of the current GPU,
 * measured with CUDA events on the caller's stream.  The float64 stencil
 * kernels are bound by this rate on GB300 (about two float64 operations per
 * clock per SM), so it is the denominator of their compute roofline.  No
 * counterpart in the reference (which has no device code).
 */
#include <cuda_runtime.h>

#include <string>

#include "prml_internal.h"

namespace {

/* Eight independent multiply-add chains per thread keep the float64 pipe
 * busy without any memory traffic; the result is stored only under a
 * condition that never holds, so the chains are not optimised away. */
__global__ void fma_chains(double* sink, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = __fma_rn(x0, a, b);
    x1 = __fma_rn(x1, a, b);
    x2 = __fma_rn(x2, a, b);
    x3 = __fma_rn(x3, a, b);
    x4 = __fma_rn(x4, a, b);
    x5 = __fma_rn(x5, a, b);
    x6 = __fma_rn(x6, a, b);
    x7 = __fma_rn(x7, a, b);
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == -12345.0) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int cuda_fail(const char* what, cudaError_t e) {
  return prml_set_error(PRML_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" int prml_measure_fp64_fma(double* fma_per_s, void* stream) {
  if (!fma_per_s) return prml_set_error(PRML_ERR_ARG, "prml_measure_fp64_fma: null output");
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail("prml_measure_fp64_fma", e);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int block = 256, grid = sms * 8, iters = 4096;
  cudaEvent_t a = nullptr, b = nullptr;
  if ((e = cudaEventCreate(&a)) != cudaSuccess || (e = cudaEventCreate(&b)) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return cuda_fail("prml_measure_fp64_fma: event", e);
  }
  float best_ms = 1e30f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    /* the first round warms the clocks up and is discarded */
    fma_chains<<<grid, block, 0, s>>>(nullptr, rep == 0 ? 64 : iters, 1.0000001, 1e-9);
    if ((e = cudaEventRecord(a, s)) != cudaSuccess) break;
    fma_chains<<<grid, block, 0, s>>>(nullptr, iters, 1.0000001, 1e-9);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if ((e = cudaEventRecord(b, s)) != cudaSuccess) break;
    if ((e = cudaEventSynchronize(b)) != cudaSuccess) break;
    float ms = 0.0f;
    if ((e = cudaEventElapsedTime(&ms, a, b)) != cudaSuccess) break;
    if (rep > 0 && ms < best_ms) best_ms = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return cuda_fail("prml_measure_fp64_fma", e);
  *fma_per_s = 8.0 * iters * (double)grid * block / (best_ms * 1e-3);
  return PRML_OK;
}
