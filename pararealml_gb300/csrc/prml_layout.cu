/*
 * Layout conversion at the drop-in boundary.
 *
 * The reference stores a state as a C-contiguous float64 array of shape
 * (*vertices_shape, C) (pararealml/operators/fdm/fdm_operator.py:53).  The
 * device kernels use planar components with padded rows,
 * [instance][C][nx][pitch], in FP32 or FP64.  prml_pack converts the former
 * into the latter (with the precision change fused in); prml_unpack does the
 * reverse into float64.
 */
#include <cuda_runtime.h>

#include "prml_internal.h"

namespace {

template <typename S>
__global__ void pack_kernel(const double* __restrict__ src, S* __restrict__ dst, int comps, int nx,
                            int ny, int pitch, long long src_bstride, long long dst_bstride,
                            int comp) {
  const long long nv = (long long)nx * ny;
  const int b = blockIdx.y;
  const double* s = src + b * src_bstride;
  S* d = dst + b * dst_bstride;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const long long i = v / ny, j = v - i * ny;
    for (int c = 0; c < comps; ++c) {
      const double x = s[v * comps + c];
      const S hi = static_cast<S>(x);
      d[(long long)c * nx * pitch + i * pitch + j] = hi;
      /* compensated state: the rounding remainder in planes [comps, 2 comps) */
      if (comp) d[(long long)(comps + c) * nx * pitch + i * pitch + j] = static_cast<S>(x - static_cast<double>(hi));
    }
  }
}

template <typename S>
__global__ void unpack_kernel(const S* __restrict__ src, double* __restrict__ dst, int comps,
                              int nx, int ny, int pitch, long long src_bstride,
                              long long dst_bstride, int comp) {
  const long long nv = (long long)nx * ny;
  const int b = blockIdx.y;
  const S* s = src + b * src_bstride;
  double* d = dst + b * dst_bstride;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const long long i = v / ny, j = v - i * ny;
    for (int c = 0; c < comps; ++c) {
      double x = static_cast<double>(s[(long long)c * nx * pitch + i * pitch + j]);
      if (comp) x += static_cast<double>(s[(long long)(comps + c) * nx * pitch + i * pitch + j]);
      d[v * comps + c] = x;
    }
  }
}

int check(int batch, int comps, int nx, int ny, int pitch) {
  if (batch < 1 || batch > 65535 || comps < 1 || nx < 1 || ny < 1 || pitch < ny)
    return prml_set_error(PRML_ERR_ARG, "layout: bad geometry");
  return PRML_OK;
}

int grid_x(int nx, int ny) {
  long long g = ((long long)nx * ny + 255) / 256;
  return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

}  // namespace

extern "C" {

int prml_pack(const double* src, void* dst, int elem_bytes, int batch, int comps, int nx, int ny,
              int pitch, long long src_bstride, long long dst_bstride, int comp, void* stream) {
  if (!src || !dst) return prml_set_error(PRML_ERR_ARG, "prml_pack: null buffer");
  int rc = check(batch, comps, nx, ny, pitch);
  if (rc) return rc;
  dim3 grid(grid_x(nx, ny), batch);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (elem_bytes == 4)
    pack_kernel<float><<<grid, 256, 0, s>>>(src, static_cast<float*>(dst), comps, nx, ny, pitch,
                                            src_bstride, dst_bstride, comp);
  else if (elem_bytes == 8)
    pack_kernel<double><<<grid, 256, 0, s>>>(src, static_cast<double*>(dst), comps, nx, ny, pitch,
                                             src_bstride, dst_bstride, comp);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_pack: elem_bytes must be 4 or 8");
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PRML_OK
                          : prml_set_error(PRML_ERR_CUDA, std::string("prml_pack: ") + cudaGetErrorString(e));
}

int prml_unpack(const void* src, int elem_bytes, double* dst, int batch, int comps, int nx, int ny,
                int pitch, long long src_bstride, long long dst_bstride, int comp, void* stream) {
  if (!src || !dst) return prml_set_error(PRML_ERR_ARG, "prml_unpack: null buffer");
  int rc = check(batch, comps, nx, ny, pitch);
  if (rc) return rc;
  dim3 grid(grid_x(nx, ny), batch);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (elem_bytes == 4)
    unpack_kernel<float><<<grid, 256, 0, s>>>(static_cast<const float*>(src), dst, comps, nx, ny,
                                              pitch, src_bstride, dst_bstride, comp);
  else if (elem_bytes == 8)
    unpack_kernel<double><<<grid, 256, 0, s>>>(static_cast<const double*>(src), dst, comps, nx, ny,
                                               pitch, src_bstride, dst_bstride, comp);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_unpack: elem_bytes must be 4 or 8");
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PRML_OK
                          : prml_set_error(PRML_ERR_CUDA, std::string("prml_unpack: ") + cudaGetErrorString(e));
}

}  // extern "C"

/* ---- Gaussian initial states ---------------------------------------------
 * out[b][v][c] = mult * exp(-0.5 * (c0 + |(x_v - mean) U|^2)) with, per
 * (instance b, component c), params = [mean (dim), U (dim x dim, row-major),
 * c0, mult]: the density scipy's multivariate_normal.pdf evaluates
 * (logpdf = -0.5 (rank log 2 pi + log pdet + maha), maha = sum of squares
 * of (x - mean) @ U), with U and c0 = rank log 2 pi + log pdet computed on
 * the host from the covariance's eigendecomposition as scipy does. */
namespace {

__global__ void gaussian_kernel(const double* __restrict__ x, long long nv, int dim, const double* __restrict__ prm,
                                int comps, double* __restrict__ out) {
  const int b = blockIdx.y;
  const int P = dim + dim * dim + 2;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    double xv[3];
    for (int i = 0; i < dim; ++i) xv[i] = x[v * dim + i];
    for (int c = 0; c < comps; ++c) {
      const double* g = prm + ((long long)b * comps + c) * P;
      double dev[3];
      for (int i = 0; i < dim; ++i) dev[i] = xv[i] - g[i];
      double maha = 0.0;
      for (int k = 0; k < dim; ++k) {
        double z = 0.0;
        for (int i = 0; i < dim; ++i) z = __dadd_rn(z, __dmul_rn(dev[i], g[dim + i * dim + k]));
        maha = __dadd_rn(maha, __dmul_rn(z, z));
      }
      const double logpdf = -0.5 * __dadd_rn(g[dim + dim * dim], maha);
      out[((long long)b * nv + v) * comps + c] = __dmul_rn(exp(logpdf), g[dim + dim * dim + 1]);
    }
  }
}

}  // namespace

extern "C" int prml_gaussian_states(const double* x, long long nv, int dim, const double* params, int batch,
                                    int comps, double* out, void* stream) {
  if (!x || !params || !out || nv < 1 || dim < 1 || dim > 3 || batch < 1 || batch > 65535 || comps < 1)
    return prml_set_error(PRML_ERR_ARG, "prml_gaussian_states: bad argument");
  const long long blocks = (nv + 255) / 256;
  dim3 grid((unsigned)(blocks < 4096 ? blocks : 4096), (unsigned)batch);
  gaussian_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, nv, dim, params, comps, out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PRML_OK
                          : prml_set_error(PRML_ERR_CUDA, std::string("prml_gaussian_states: ") + cudaGetErrorString(e));
}
