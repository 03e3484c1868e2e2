/*
 * Implicit integrators: backward Euler and Crank-Nicolson with the
 * element-wise secant solve of the reference.
 *
 * Reference: BackwardEulerMethod / CrankNicolsonMethod.integral and
 * ImplicitMethod._solve (pararealml/operators/fdm/numerical_integrator.py:
 * 135-270).  The step solves, for y_next,
 *
 *   y_next - c(y + a dt f(t + dt, y_next) + (1 - a) dt f(t, y)) = 0
 *
 * (backward Euler: y_next - c(y + dt f(t + dt, y_next))) with
 * scipy.optimize.newton and no derivative, i.e. the secant method applied
 * element by element to the whole array: starting from p = c(y + dt f(t, y))
 * and p1 = p (1 + dx) +- dx (dx = eps^0.33), every element with q1 != q0 steps
 * to p1 - q1 (p1 - p) / (q1 - q0); elements whose residuals are equal are set
 * once to the midpoint (p1 + p) / 2 and then stay; the loop stops when every
 * element that stepped moved by less than tol, when no residual changed
 * (all elements to the midpoint), or after max_iterations steps.
 *
 * The kernels here are the element-wise parts (float64, rounded like the
 * numpy expressions: no contraction, IEEE division); the right-hand sides
 * come from the generated stencil module (prml_fdm_rhs).  Each instance
 * stops on its own counters, as separate reference solves would: the stop
 * test, the result copy and the status sums run on the device
 * (prml_implicit_stop, which also counts the iterations in device memory),
 * so the host can issue several iterations (or replay them as a CUDA graph)
 * before it reads whether every instance has finished; iterations of
 * finished instances leave them unchanged.
 */
#include <cuda_runtime.h>

#include <string>

#include "prml_internal.h"

namespace {

constexpr int IT = 256;

enum { C_CHANGED = 0, C_FAILING = 1, C_FLAT = 2, C_DONE = 3 };
enum { F_FAIL = 1, F_ACTIVE = 2, F_NZ = 4 };

/* element (b, c, row, col) of the planar state from a grid-stride index over
 * [batch][C][rows][pitch]; false for padding columns */
struct Elem {
  int b, c, row, col;
  long long off;
};

__device__ __forceinline__ bool elem_of(const prml_implicit_params& p, long long e, int rows, Elem& q) {
  const long long plane = (long long)rows * p.pitch;
  q.b = (int)(e / p.inst);
  const long long r = e - (long long)q.b * p.inst;
  q.c = (int)(r / plane);
  const long long r2 = r - (long long)q.c * plane;
  q.row = (int)(r2 / p.pitch);
  q.col = (int)(r2 - (long long)q.row * p.pitch);
  q.off = e;
  return q.col < p.n[2] && q.c < p.comps;
}

/* Dirichlet value of component c at the vertex of storage row `row`,
 * column j (faces in axis order, lower then upper: later axes win at edges
 * and corners); v unchanged where no value is given. */
__device__ __forceinline__ double dirichlet(const prml_implicit_params& p, double v, int c, int row, int j) {
  if (!p.dirichlet) return v;
  const int z = row / p.n[1], i = row - z * p.n[1];
  const int q[3] = {z, i, j};
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const int ka = f >> 1;
    if (ka < p.first_axis) continue;
    if (q[ka] != ((f & 1) ? p.n[ka] - 1 : 0)) continue;
    const int tf = f - p.face_base;
    if (tf < 0 || !((p.dir_mask >> (tf * p.comps + c)) & 1ull)) continue;
    const int idx = ka == 0 ? i * p.n[2] + j : (ka == 1 ? z * p.n[2] + j : z * p.n[1] + i);
    const double d = p.dirichlet[((long long)tf * p.comps + c) * p.face_len + idx];
    if (d == d) v = d;
  }
  return v;
}

__device__ __forceinline__ bool is_d(const prml_implicit_params& p, int c) { return (p.d_mask >> c) & 1ull; }

__global__ void predict_kernel(const prml_implicit_params p, int rows, long long n, const double* __restrict__ y,
                               const double* __restrict__ f, double* __restrict__ fu, double* __restrict__ x0,
                               double* __restrict__ x1, unsigned char* __restrict__ flags,
                               const int* __restrict__ counters) {
  const double dx = p.dx;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    Elem q;
    if (!elem_of(p, e, rows, q) || counters[4 * q.b + C_DONE]) continue;
    const double u = is_d(p, q.c) ? __dmul_rn(p.dt, f[e]) : 0.0;
    fu[e] = u;
    const double v = dirichlet(p, __dadd_rn(y[e], u), q.c, q.row, q.col);
    x0[e] = v;
    x1[e] = __dadd_rn(__dmul_rn(v, __dadd_rn(1.0, dx)), v >= 0.0 ? dx : -dx);
    flags[e] = F_FAIL | F_ACTIVE;
  }
}

__global__ void residual_kernel(const prml_implicit_params p, int rows, long long n, const double* __restrict__ x,
                                const double* __restrict__ y, const double* __restrict__ f,
                                const double* __restrict__ fu, double* __restrict__ qout,
                                const double* __restrict__ q_prev, int* __restrict__ counters) {
  const double adt = __dmul_rn(p.a, p.dt);
  const double b = 1.0 - p.a;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    Elem q;
    if (!elem_of(p, e, rows, q) || counters[4 * q.b + C_DONE]) continue;
    const double fv = is_d(p, q.c) ? f[e] : 0.0;
    double s;
    if (p.crank_nicolson) /* y + a * dt * f + b * forward_update */
      s = __dadd_rn(__dadd_rn(y[e], __dmul_rn(adt, fv)), __dmul_rn(b, fu[e]));
    else /* y + dt * f */
      s = __dadd_rn(y[e], __dmul_rn(p.dt, fv));
    const double r = __dsub_rn(x[e], dirichlet(p, s, q.c, q.row, q.col));
    qout[e] = r;
    if (q_prev && r != q_prev[e]) counters[4 * q.b + C_CHANGED] = 1;
  }
}

__global__ void update_kernel(const prml_implicit_params p, int rows, long long n, double* __restrict__ x0,
                              const double* __restrict__ x1, const double* __restrict__ q0,
                              const double* __restrict__ q1, unsigned char* __restrict__ flags,
                              int* __restrict__ counters) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    Elem q;
    if (!elem_of(p, e, rows, q) || counters[4 * q.b + C_DONE]) continue;
    const double a0 = x0[e], a1 = x1[e];
    unsigned char fl = flags[e];
    if (!counters[4 * q.b + C_CHANGED]) {
      /* no residual of the instance changed: every element to the midpoint */
      x0[e] = __ddiv_rn(__dadd_rn(a1, a0), 2.0);
      fl &= (unsigned char)~F_NZ;
      flags[e] = fl;
      counters[4 * q.b + C_FLAT] = 1;
      continue;
    }
    const double r0 = q0[e], r1 = q1[e];
    if (r1 != r0) {
      const double step = __ddiv_rn(__dmul_rn(r1, __dsub_rn(a1, a0)), __dsub_rn(r1, r0));
      x0[e] = __dsub_rn(a1, step);
      const bool fail = fabs(step) >= p.tol;
      fl = (unsigned char)((fl & F_ACTIVE) | F_NZ | (fail ? F_FAIL : 0));
      if (fail) counters[4 * q.b + C_FAILING] = 1;
    } else {
      if (fl & F_ACTIVE) x0[e] = __ddiv_rn(__dadd_rn(a1, a0), 2.0);
      fl = (unsigned char)(fl & F_FAIL);  /* inactive from now on, failure state kept */
    }
    flags[e] = fl;
  }
}

__global__ void status_kernel(const prml_implicit_params p, int rows, long long n, const double* __restrict__ x0,
                              const double* __restrict__ x1, const unsigned char* __restrict__ flags,
                              double* __restrict__ out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    Elem q;
    if (!elem_of(p, e, rows, q)) continue;
    const unsigned char fl = flags[e];
    const bool fail = fl & F_FAIL;
    atomicAdd(out + 4 * q.b + 1, 1.0);
    if (fail) {
      atomicAdd(out + 4 * q.b + 0, 1.0);
      if (!(fl & F_NZ)) {
        atomicAdd(out + 4 * q.b + 2, 1.0);
        const double d = x1[e] - x0[e];
        if (x1[e] != x0[e]) atomicAdd(out + 4 * q.b + 3, d * d);
      }
    }
  }
}

__global__ void finish_kernel(const prml_implicit_params p, int rows, long long n, const double* __restrict__ x,
                              const double* __restrict__ f, double* __restrict__ out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    Elem q;
    if (!elem_of(p, e, rows, q)) continue;
    out[e] = is_d(p, q.c) ? x[e] : dirichlet(p, f[e], q.c, q.row, q.col);
  }
}

/* An instance stops at this iteration when every element that stepped
 * moved by less than tol (no failing counter) or no residual changed (all
 * to the midpoint); with `force` every instance still running stops (the
 * iteration limit).  Finished instances never stop again. */
__device__ __forceinline__ bool stops_now(const int* __restrict__ counters, int b, int force) {
  const int* c = counters + 4 * b;
  return !c[C_DONE] && (force || c[C_FLAT] || !c[C_FAILING]);
}

/* For the instances that stop now: their result is xs, and their status
 * (the sums of status_kernel over x0 = xs, x1 = xo) is added to stats. */
__global__ void stop_kernel(const prml_implicit_params p, int rows, long long n, const double* __restrict__ xs,
                            const double* __restrict__ xo, const unsigned char* __restrict__ flags,
                            const int* __restrict__ counters, int force, double* __restrict__ res,
                            double* __restrict__ stats) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(e / p.inst);
    if (!stops_now(counters, b, force)) continue;
    res[e] = xs[e];
    Elem q;
    if (!elem_of(p, e, rows, q)) continue;
    const unsigned char fl = flags[e];
    atomicAdd(stats + 4 * b + 1, 1.0);
    if (fl & F_FAIL) {
      atomicAdd(stats + 4 * b + 0, 1.0);
      if (!(fl & F_NZ)) {
        atomicAdd(stats + 4 * b + 2, 1.0);
        const double d = xo[e] - xs[e];
        if (xo[e] != xs[e]) atomicAdd(stats + 4 * b + 3, d * d);
      }
    }
  }
}

/* After stop_kernel (one block): the iteration counter advances (a forced
 * stop closes the iteration the counter already names), the instances that
 * stopped are finished at that iteration, and every instance's
 * per-iteration counters are cleared for the next residual and update. */
__global__ void mark_kernel(int batch, int* __restrict__ counters, int force, int* __restrict__ iteration,
                            int* __restrict__ iterations) {
  const int it = *iteration + (force ? 0 : 1);
  for (int b = threadIdx.x; b < batch; b += blockDim.x) {
    if (stops_now(counters, b, force)) {
      counters[4 * b + C_DONE] = 1;
      iterations[b] = it;
    }
    counters[4 * b + C_CHANGED] = 0;
    counters[4 * b + C_FAILING] = 0;
    counters[4 * b + C_FLAT] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) *iteration = it;
}

int check(const prml_implicit_params* p) {
  if (!p) return prml_set_error(PRML_ERR_ARG, "implicit: null parameters");
  if (p->batch < 1 || p->comps < 1 || p->comps > 64 || p->pitch < p->n[2])
    return prml_set_error(PRML_ERR_ARG, "implicit: bad shape");
  if (p->first_axis < 0 || p->first_axis > 3) return prml_set_error(PRML_ERR_ARG, "implicit: bad first_axis");
  for (int a = 0; a < 3; ++a)
    if (p->n[a] < 1) return prml_set_error(PRML_ERR_ARG, "implicit: bad mesh extent");
  if (!(p->a >= 0.0 && p->a <= 1.0)) return prml_set_error(PRML_ERR_ARG, "the value of 'a' must be between 0 and 1");
  if (p->tol < 0.0) return prml_set_error(PRML_ERR_ARG, "tolerance must be non-negative");
  if (!(p->dx > 0.0)) return prml_set_error(PRML_ERR_ARG, "implicit: bad secant offset");
  if (p->cstride < (long long)p->n[0] * p->n[1] * p->pitch || p->inst < p->cstride * p->comps)
    return prml_set_error(PRML_ERR_ARG, "implicit: bad strides");
  return PRML_OK;
}

long long elems(const prml_implicit_params* p) { return p->inst * p->batch; }
int rows_of(const prml_implicit_params* p) { return p->n[0] * p->n[1]; }
int grid_of(long long n) {
  long long g = (n + IT - 1) / IT;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

int last(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return PRML_OK;
}

}  // namespace

extern "C" {

int prml_implicit_params_size(void) { return (int)sizeof(prml_implicit_params); }

int prml_implicit_predict(const prml_implicit_params* p, const double* y, const double* f, double* fu, double* x0,
                          double* x1, unsigned char* flags, int* counters, void* stream) {
  int rc = check(p);
  if (rc) return rc;
  if (!y || !f || !fu || !x0 || !x1 || !flags || !counters) return prml_set_error(PRML_ERR_ARG, "implicit_predict: null buffer");
  const long long n = elems(p);
  predict_kernel<<<grid_of(n), IT, 0, static_cast<cudaStream_t>(stream)>>>(*p, rows_of(p), n, y, f, fu, x0, x1, flags,
                                                                          counters);
  return last("implicit_predict");
}

int prml_implicit_residual(const prml_implicit_params* p, const double* x, const double* y, const double* f,
                           const double* fu, double* q, const double* q_prev, int* counters, void* stream) {
  int rc = check(p);
  if (rc) return rc;
  if (!x || !y || !f || !fu || !q || !counters) return prml_set_error(PRML_ERR_ARG, "implicit_residual: null buffer");
  const long long n = elems(p);
  residual_kernel<<<grid_of(n), IT, 0, static_cast<cudaStream_t>(stream)>>>(*p, rows_of(p), n, x, y, f, fu, q, q_prev,
                                                                           counters);
  return last("implicit_residual");
}

int prml_implicit_update(const prml_implicit_params* p, double* x0, const double* x1, const double* q0,
                         const double* q1, unsigned char* flags, int* counters, void* stream) {
  int rc = check(p);
  if (rc) return rc;
  if (!x0 || !x1 || !q0 || !q1 || !flags || !counters) return prml_set_error(PRML_ERR_ARG, "implicit_update: null buffer");
  const long long n = elems(p);
  update_kernel<<<grid_of(n), IT, 0, static_cast<cudaStream_t>(stream)>>>(*p, rows_of(p), n, x0, x1, q0, q1, flags,
                                                                         counters);
  return last("implicit_update");
}

int prml_implicit_status(const prml_implicit_params* p, const double* x0, const double* x1,
                         const unsigned char* flags, double* out, void* stream) {
  int rc = check(p);
  if (rc) return rc;
  if (!x0 || !x1 || !flags || !out) return prml_set_error(PRML_ERR_ARG, "implicit_status: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * 4 * p->batch, s);
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("implicit_status: ") + cudaGetErrorString(e));
  const long long n = elems(p);
  status_kernel<<<grid_of(n), IT, 0, s>>>(*p, rows_of(p), n, x0, x1, flags, out);
  return last("implicit_status");
}

int prml_implicit_stop(const prml_implicit_params* p, const double* xs, const double* xo,
                       const unsigned char* flags, int* counters, int* iteration, int force, double* res,
                       double* stats, int* iterations, void* stream) {
  int rc = check(p);
  if (rc) return rc;
  if (!xs || !xo || !flags || !counters || !iteration || !res || !stats || !iterations)
    return prml_set_error(PRML_ERR_ARG, "implicit_stop: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long n = elems(p);
  stop_kernel<<<grid_of(n), IT, 0, s>>>(*p, rows_of(p), n, xs, xo, flags, counters, force ? 1 : 0, res, stats);
  rc = last("implicit_stop");
  if (rc) return rc;
  mark_kernel<<<1, IT, 0, s>>>(p->batch, counters, force ? 1 : 0, iteration, iterations);
  return last("implicit_stop(mark)");
}

int prml_implicit_finish(const prml_implicit_params* p, const double* x, const double* f, double* out,
                         void* stream) {
  int rc = check(p);
  if (rc) return rc;
  if (!x || !f || !out) return prml_set_error(PRML_ERR_ARG, "implicit_finish: null buffer");
  const long long n = elems(p);
  finish_kernel<<<grid_of(n), IT, 0, static_cast<cudaStream_t>(stream)>>>(*p, rows_of(p), n, x, f, out);
  return last("implicit_finish");
}

}  // extern "C"
