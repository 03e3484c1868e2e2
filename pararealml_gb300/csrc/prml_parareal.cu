/*
 * Parareal correction kernels (FP64) for batched, single-GPU Parareal.
 *
 * Reference: pararealml/operators/parareal/parareal_operator.py:102-197.
 * There, each MPI rank owns one time slice; after the fine solves the ranks
 * allgather the corrections F(U_j) - G_old(U_j) (:164-165) and every rank
 * replays the sequential coarse sweep U_{j+1} = G(U_j) + correction_j
 * (:167-185).  Here all slices (and all initial conditions of an ensemble)
 * live in one device array, so the allgather is just a device-memory write
 * and the sweep is a chain of launches on one stream.
 *
 * Buffers: border points U are FP64 [slice][instance][C][nx][pitch]; fine and
 * coarse solver states are FP32 or FP64 ("state" type, elem_bytes 4 or 8) in
 * the same layout.  All counts are in elements.  `active` (nullable) masks
 * instances that have already met their termination condition: their
 * border points are left untouched, which is what the reference does for a
 * problem whose loop has exited.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "prml_internal.h"

/* Fixed scratch of prml_pr_update_norm_noalloc (see the header): the
 * partial sums of the norm live here instead of in a caller buffer.  Every
 * GPU that loads this library holds the array until the process exits. */
static __device__ __align__(256) double g_noalloc_norm_partial[PRML_NOALLOC_NORM_SCRATCH_ELEMS];

namespace {

/* Device address of g_noalloc_norm_partial per device, with the context it
 * was resolved in: a device reset (or any teardown and re-creation of the
 * primary context) reloads the module at another address, so the address
 * is looked up again whenever the current context differs. */
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[PRML_NOALLOC_MAX_DEVICES] = {nullptr};
void* g_noalloc_ctx[PRML_NOALLOC_MAX_DEVICES] = {nullptr};

/* Element i of a float64 buffer and its counterpart in a state buffer.
 * Plain states (ce == 0) share the float64 layout.  Compensated states hold
 * each instance's ce leading ("hi") words followed by ce trailing ("lo")
 * words; the value is hi + lo. */
__device__ __forceinline__ long long hi_index(long long i, long long ce) {
  if (ce == 0) return i;
  const long long inst = i / ce;
  return inst * 2 * ce + (i - inst * ce);
}

template <typename S>
__device__ __forceinline__ double load_state(const S* s, long long i, long long ce) {
  const long long h = hi_index(i, ce);
  double v = static_cast<double>(s[h]);
  if (ce) v += static_cast<double>(s[h + ce]);
  return v;
}

template <typename S>
__device__ __forceinline__ void store_state(S* s, long long i, long long ce, double v) {
  const long long h = hi_index(i, ce);
  const S hi = static_cast<S>(v);
  s[h] = hi;
  if (ce) s[h + ce] = static_cast<S>(v - static_cast<double>(hi));
}

template <typename S>
__global__ void cast_from_f64(const double* __restrict__ src, S* __restrict__ dst, long long n,
                              long long ce) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    store_state(dst, i, ce, src[i]);
}

template <typename S>
__global__ void correct(const S* __restrict__ fine_end, const double* __restrict__ coarse_old,
                        double* __restrict__ corr, long long n, long long per_instance,
                        const int* __restrict__ active, int batch, long long ce) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (active) {
      const int b = (int)((i / per_instance) % batch);
      if (!active[b]) continue;
    }
    corr[i] = load_state(fine_end, i, ce) - coarse_old[i];
  }
}

/* coarse_store = coarse_new (if given); u_next = coarse_store + corr;
 * u_next_state = state-typed copy of u_next (if given). */
template <typename S>
__global__ void advance(const S* __restrict__ coarse_new, double* __restrict__ coarse_store,
                        const double* __restrict__ corr, double* __restrict__ u_next,
                        S* __restrict__ u_next_state, long long n, long long per_instance,
                        const int* __restrict__ active, int batch, long long ce) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (active) {
      const int b = (int)((i / per_instance) % batch);
      if (!active[b]) continue;
    }
    double g = coarse_store[i];
    if (coarse_new) {
      g = load_state(coarse_new, i, ce);
      coarse_store[i] = g;
    }
    const double u = g + corr[i];
    u_next[i] = u;
    if (u_next_state) store_state(u_next_state, i, ce, u);
  }
}

/* partial[(plane)*chunks + chunk] = sum over the chunk of (a - b)^2, where a
 * plane is one component of one instance of one slice (nx x ny vertices,
 * rows `pitch` apart). */
__global__ void sq_diff_partial(const double* __restrict__ a, const double* __restrict__ b,
                                int nx, int ny, int pitch, int chunks,
                                double* __restrict__ partial) {
  const long long plane = blockIdx.y;
  const long long base = plane * (long long)nx * pitch;
  const long long nv = (long long)nx * ny;
  const long long per = (nv + chunks - 1) / chunks;
  const long long lo = blockIdx.x * per;
  const long long hi = lo + per < nv ? lo + per : nv;
  double s = 0.0;
  for (long long v = lo + threadIdx.x; v < hi; v += blockDim.x) {
    const long long r = v / ny, c = v - r * ny;
    const double d = a[base + r * pitch + c] - b[base + r * pitch + c];
    s += d * d;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) partial[plane * chunks + blockIdx.x] = s;
  }
}

/* out[b*C + c] = max over slices j of sqrt(mean over vertices of (a-b)^2). */
__global__ void rms_max(const double* __restrict__ partial, int slices, int batch, int comps,
                        int chunks, long long nv, double* __restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= batch * comps) return;
  const int b = idx / comps, c = idx - b * comps;
  double best = 0.0;
  for (int j = 0; j < slices; ++j) {
    const long long plane = ((long long)j * batch + b) * comps + c;
    double s = 0.0;
    for (int k = 0; k < chunks; ++k) s += partial[plane * chunks + k];
    const double rms = sqrt(s / (double)nv);
    /* np.maximum: a NaN RMS makes the maximum NaN (and it stays NaN) */
    best = (rms > best || rms != rms) ? rms : best;
  }
  out[idx] = best;
}

__global__ void masked_copy(const double* __restrict__ src, double* __restrict__ dst, long long n,
                            long long per_instance, const int* __restrict__ active, int batch) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (active) {
      const int b = (int)((i / per_instance) % batch);
      if (!active[b]) continue;
    }
    dst[i] = src[i];
  }
}

/* delta = u_end - end_state (state type promoted to double) */
template <typename S>
__global__ void end_delta(const double* __restrict__ u_end, const S* __restrict__ end_state,
                          double* __restrict__ delta, long long n, long long ce) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    delta[i] = u_end[i] - load_state(end_state, i, ce);
}

int grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g < 1 ? 1 : g);
}

int last_cuda(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return PRML_OK;
}

}  // namespace

extern "C" {

int prml_pr_cast(const double* src, void* dst, int elem_bytes, long long n, long long comp,
                 void* stream) {
  if (!src || !dst || n < 0 || comp < 0) return prml_set_error(PRML_ERR_ARG, "prml_pr_cast: bad argument");
  if (n == 0) return PRML_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (elem_bytes == 4)
    cast_from_f64<float><<<grid_for(n), 256, 0, s>>>(src, static_cast<float*>(dst), n, comp);
  else if (elem_bytes == 8)
    cast_from_f64<double><<<grid_for(n), 256, 0, s>>>(src, static_cast<double*>(dst), n, comp);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_pr_cast: elem_bytes must be 4 or 8");
  return last_cuda("prml_pr_cast");
}

int prml_pr_correct(const void* fine_end, int elem_bytes, const double* coarse_old, double* corr,
                    long long n, long long per_instance, const int* active, int batch,
                    long long comp, void* stream) {
  if (!fine_end || !coarse_old || !corr || n < 0 || per_instance < 1 || batch < 1 || comp < 0)
    return prml_set_error(PRML_ERR_ARG, "prml_pr_correct: bad argument");
  if (n == 0) return PRML_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (elem_bytes == 4)
    correct<float><<<grid_for(n), 256, 0, s>>>(static_cast<const float*>(fine_end), coarse_old,
                                               corr, n, per_instance, active, batch, comp);
  else if (elem_bytes == 8)
    correct<double><<<grid_for(n), 256, 0, s>>>(static_cast<const double*>(fine_end), coarse_old,
                                                corr, n, per_instance, active, batch, comp);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_pr_correct: elem_bytes must be 4 or 8");
  return last_cuda("prml_pr_correct");
}

int prml_pr_advance(const void* coarse_new, int elem_bytes, double* coarse_store,
                    const double* corr, double* u_next, void* u_next_state, long long n,
                    long long per_instance, const int* active, int batch, long long comp,
                    void* stream) {
  if (!coarse_store || !corr || !u_next || n < 0 || per_instance < 1 || batch < 1 || comp < 0)
    return prml_set_error(PRML_ERR_ARG, "prml_pr_advance: bad argument");
  if (n == 0) return PRML_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (elem_bytes == 4)
    advance<float><<<grid_for(n), 256, 0, s>>>(static_cast<const float*>(coarse_new),
                                               coarse_store, corr, u_next,
                                               static_cast<float*>(u_next_state), n,
                                               per_instance, active, batch, comp);
  else if (elem_bytes == 8)
    advance<double><<<grid_for(n), 256, 0, s>>>(static_cast<const double*>(coarse_new),
                                                coarse_store, corr, u_next,
                                                static_cast<double*>(u_next_state), n,
                                                per_instance, active, batch, comp);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_pr_advance: elem_bytes must be 4 or 8");
  return last_cuda("prml_pr_advance");
}

int prml_pr_copy(const double* src, double* dst, long long n, long long per_instance,
                 const int* active, int batch, void* stream) {
  if (!src || !dst || n < 0 || per_instance < 1 || batch < 1)
    return prml_set_error(PRML_ERR_ARG, "prml_pr_copy: bad argument");
  if (n == 0) return PRML_OK;
  masked_copy<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(src, dst, n, per_instance,
                                                                          active, batch);
  return last_cuda("prml_pr_copy");
}

int prml_pr_end_delta(const double* u_end, const void* end_state, int elem_bytes, double* delta,
                      long long n, long long comp, void* stream) {
  if (!u_end || !end_state || !delta || n < 0 || comp < 0)
    return prml_set_error(PRML_ERR_ARG, "prml_pr_end_delta: bad argument");
  if (n == 0) return PRML_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (elem_bytes == 4)
    end_delta<float><<<grid_for(n), 256, 0, s>>>(u_end, static_cast<const float*>(end_state), delta, n, comp);
  else if (elem_bytes == 8)
    end_delta<double><<<grid_for(n), 256, 0, s>>>(u_end, static_cast<const double*>(end_state), delta, n, comp);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_pr_end_delta: elem_bytes must be 4 or 8");
  return last_cuda("prml_pr_end_delta");
}

long long prml_pr_norm_scratch_elems(int slices, int batch, int comps, int chunks) {
  return (long long)slices * batch * comps * chunks;
}

int prml_pr_update_norm(const double* new_pts, const double* old_pts, int slices, int batch,
                        int comps, int nx, int ny, int pitch, int chunks, double* partial,
                        double* out, void* stream) {
  if (!new_pts || !old_pts || !partial || !out || slices < 1 || batch < 1 || comps < 1 ||
      nx < 1 || ny < 1 || pitch < ny || chunks < 1)
    return prml_set_error(PRML_ERR_ARG, "prml_pr_update_norm: bad argument");
  const long long planes = (long long)slices * batch * comps;
  if (planes > 65535) return prml_set_error(PRML_ERR_ARG, "prml_pr_update_norm: too many planes");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  sq_diff_partial<<<dim3(chunks, (unsigned)planes), 256, 0, s>>>(new_pts, old_pts, nx, ny, pitch,
                                                                 chunks, partial);
  int rc = last_cuda("prml_pr_update_norm(partial)");
  if (rc) return rc;
  const int n = batch * comps;
  rms_max<<<(n + 127) / 128, 128, 0, s>>>(partial, slices, batch, comps, chunks,
                                          (long long)nx * ny, out);
  return last_cuda("prml_pr_update_norm(max)");
}

int prml_pr_update_norm_noalloc(const double* new_pts, const double* old_pts, int slices,
                                int batch, int comps, int nx, int ny, int pitch, int chunks,
                                double* out, void* stream) {
  if (!new_pts || !old_pts || !out || slices < 1 || batch < 1 || comps < 1 || nx < 1 ||
      ny < 1 || pitch < ny || chunks < 1)
    return prml_set_error(PRML_ERR_ARG, "prml_pr_update_norm_noalloc: bad argument");
  const long long need = (long long)slices * batch * comps * chunks;
  if (need > PRML_NOALLOC_NORM_SCRATCH_ELEMS)
    return prml_set_error(PRML_ERR_ARG,
                          "prml_pr_update_norm_noalloc: slices*batch*comps*chunks = " +
                              std::to_string(need) + " exceeds its fixed scratch of " +
                              std::to_string(PRML_NOALLOC_NORM_SCRATCH_ELEMS) +
                              " doubles; use fewer chunks or prml_pr_update_norm");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return prml_set_error(PRML_ERR_CUDA, std::string("prml_pr_update_norm_noalloc: cudaGetDevice: ") +
                                             cudaGetErrorString(e));
  if (dev < 0 || dev >= PRML_NOALLOC_MAX_DEVICES)
    return prml_set_error(PRML_ERR_ARG, "prml_pr_update_norm_noalloc: device ordinal out of range");
  double* partial = nullptr;
  {
    /* first call on this device: look up the array's device address while
     * the device is current (the name is only a host-side stand-in) */
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    void* ctx = prml_current_context();
    if (!g_noalloc_ptr[dev] || ctx != g_noalloc_ctx[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_norm_partial);
      if (e != cudaSuccess || !p)
        return prml_set_error(PRML_ERR_CUDA,
                              std::string("prml_pr_update_norm_noalloc: cudaGetSymbolAddress: ") +
                                  cudaGetErrorString(e));
      g_noalloc_ptr[dev] = static_cast<double*>(p);
      /* the runtime call above made the device's primary context current */
      g_noalloc_ctx[dev] = prml_current_context();
    }
    partial = g_noalloc_ptr[dev];
  }
  /* every partial slot the second kernel reads is written by the first one
   * in this same call, so nothing left by an earlier call is ever read */
  const long long planes = (long long)slices * batch * comps;
  if (planes > 65535) return prml_set_error(PRML_ERR_ARG, "prml_pr_update_norm_noalloc: too many planes");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  sq_diff_partial<<<dim3(chunks, (unsigned)planes), 256, 0, s>>>(new_pts, old_pts, nx, ny, pitch,
                                                                 chunks, partial);
  int rc = last_cuda("prml_pr_update_norm_noalloc(partial)");
  if (rc) return rc;
  const int n = batch * comps;
  rms_max<<<(n + 127) / 128, 128, 0, s>>>(partial, slices, batch, comps, chunks,
                                          (long long)nx * ny, out);
  return last_cuda("prml_pr_update_norm_noalloc(max)");
}

}  // extern "C"
