/*
 * Anti-Laplacian by Jacobi iteration: the solve FDMOperator runs once per
 * step for the LHS.Y_LAPLACIAN components (the stream function of the
 * reference's Navier-Stokes system).
 *
 * Reference: NumericalDifferentiator.anti_laplacian and
 * ThreePointCentralDifferenceMethod._next_anti_laplacian_estimate /
 * _add_halos_along_axis (pararealml/operators/fdm/numerical_differentiator.py:
 * 872-927, 1097-1186, 1188-1242).  Per iteration and vertex:
 *
 *   acc   = sum over mesh axes of (prev + next) / dx^2 (+ the curvilinear
 *           first-derivative terms and 1/r^2, 1/(r sin phi)^2 factors)
 *   y_new = (acc - laplacian) / denominator
 *
 * with ghost vertices y[1] - 2 dx g (lower) and y[n-2] + 2 dx g (upper) where
 * a Neumann value g is given, zero where none is, then the Dirichlet values
 * re-imposed (later axes win at corners, constrained_problem.py:262-301).
 * The loop stops after the first iteration whose change has a 2-norm, over
 * all solved components of the instance, of at most tol (the reference's
 * `while diff > tol`, so a NaN change also stops it).  Divisions by the
 * step sizes and denominators are products with host-computed reciprocals.
 *
 * One cooperative launch per solve: the CTAs of an instance split its
 * (component, vertex) items, two ping-pong buffers hold the estimates, and
 * one grid barrier per iteration separates the iterations.  Every CTA sums
 * the per-CTA partial norms in the same order, so all CTAs take the same
 * stop decision for every instance without any host round trip.  The
 * barrier wait is bounded (2 s of %globaltimer); on expiry the kernel
 * records status 2 and every CTA leaves at its next barrier.
 */
#include <cuda_runtime.h>

#include <string>

#include "prml_internal.h"

namespace {

constexpr int JT = 256;  // threads per CTA of the unstaged kernel
constexpr int JS = 512;  // threads per CTA of the staged kernel
constexpr unsigned long long BARRIER_NS = 2000000000ull;

/* Scratch layout (bytes, each part 256-byte aligned):
 *   control: [0] barrier arrivals (u64, counts up through the whole launch),
 *            [64] release word of the staged kernel's barrier (u64),
 *            [128] status (u32); each on its own 64-byte line
 *   dec:     int per instance: the staged kernel's stop decision
 *   iters:   long long per instance (iterations, -1 = not converged)
 *   partial: double [2][8][batch][G] (parity, iteration of the block, instance, CTA)
 *   buffers: two estimates [batch][n_lap][V] in the state type */
struct Layout {
  long long control, iters, dec, partial, buf0, buf1, total;
};

long long align256(long long x) { return (x + 255) / 256 * 256; }

Layout layout_of(const prml_jacobi_params& p, int G) {
  const long long V = (long long)p.n[0] * p.n[1] * p.n[2];
  Layout L;
  L.control = 0;
  L.iters = 256;
  L.dec = L.iters + align256(8LL * p.batch);
  L.partial = L.dec + align256(4LL * p.batch);
  L.buf0 = L.partial + align256(8LL * 2 * 8 * p.batch * G);
  const long long buf = align256((long long)p.elem_bytes * p.batch * p.n_lap * V);
  L.buf1 = L.buf0 + buf;
  L.total = L.buf1 + buf;
  return L;
}

/* floor(a / d) for 0 <= a < 2^31 by multiply and shift (Granlund and
 * Montgomery, "Division by invariant integers using multiplication", 1994):
 * l = ceil(log2 d), m = floor(2^(32 + l) / d) + 1. */
struct Div {
  unsigned long long m;
  int shift;
  int d;
};

Div make_div(int d) {
  int l = 0;
  while ((1LL << l) < d) ++l;
  Div r;
  r.m = (unsigned long long)(((__uint128_t)1 << (32 + l)) / (unsigned)d) + 1ull;
  r.shift = 32 + l;
  r.d = d;
  return r;
}

__device__ __forceinline__ int div_(int a, const Div& q) {
  return (int)(((unsigned long long)(unsigned)a * q.m) >> q.shift);
}

/* Per-launch constants of the kernel (by value, kept in registers). */
template <typename T>
struct Geo {
  int n[3];
  int V;
  int stride[3];  // dense strides of the kernel axes
  T inv_dxx[3], two_dx[3];
  Div d12, d2;    // division by n[1] * n[2] and by n[2]
  const T* dir;
  const T* neu;
  unsigned long long dmask, nmask;
  int comps, flen, fbase;
  int pitch;
  long long cstride;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* a) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
  return v;
}

__device__ __forceinline__ unsigned ld_acquire32(const unsigned* a) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
  return v;
}

/* Grid-wide barrier: one arrival per CTA on a counter that only grows
 * within the launch; barrier k is passed once it reads k * gridDim.x.  The
 * wait is bounded.  Single-CTA grids only need the CTA barrier. */
__device__ __forceinline__ void grid_sync(unsigned long long* cnt, unsigned* status, unsigned long long& target) {
  __syncthreads();
  if (gridDim.x == 1) return;
  target += gridDim.x;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(cnt, 1ull);
    const unsigned long long t0 = global_ns();
    while (ld_acquire64(cnt) < target) {
      __nanosleep(20);
      if (global_ns() - t0 > BARRIER_NS) {
        atomicOr(status, 2u);
        break;
      }
    }
  }
  __syncthreads();
}

/* Deterministic CTA sum: per-warp shuffle tree, then warp 0 over the warps,
 * in the accumulator type A (float for float32 states: FP64 issues at a
 * small fraction of the FP32 rate on this GPU); red holds NT / 32 values of
 * A.  The result is valid in warp 0. */
template <int NT = JT, typename A>
__device__ __forceinline__ double block_sum(A v, A* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[w] = v;
  __syncthreads();
  A s = A(0);
  if (w == 0) {
    s = lane < (NT / 32) ? red[lane] : A(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return double(s);
}

/* Rounded arithmetic without contraction, so each operation rounds like
 * the reference's numpy expression. */
template <typename T> __device__ __forceinline__ T add_(T a, T b);
template <typename T> __device__ __forceinline__ T sub_(T a, T b);
template <typename T> __device__ __forceinline__ T mul_(T a, T b);
template <> __device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float sub_(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
/* a * b + c with one rounding (the squared-change sums) */
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }

/* Table index of vertex (z, i, j) on 3D-numbered face f (axis f >> 1): the
 * two other kernel axes in C order. */
__device__ __forceinline__ int face_index(int f, int z, int i, int j, const int (&n)[3]) {
  const int ka = f >> 1;
  return ka == 0 ? i * n[2] + j : (ka == 1 ? z * n[2] + j : z * n[1] + i);
}

template <typename T>
__device__ __forceinline__ bool table_value(const Geo<T>& g, const T* tab, unsigned long long mask, int f, int c,
                                            int z, int i, int j, T& out) {
  const int tf = f - g.fbase;
  if (tf < 0 || !((mask >> (tf * g.comps + c)) & 1ull)) return false;
  const T v = tab[((long long)tf * g.comps + c) * g.flen + face_index(f, z, i, j, g.n)];
  if (v != v) return false;
  out = v;
  return true;
}

/* One Jacobi estimate at dense vertex v of a solved component whose
 * estimates start at `cur`.  EDGE = false: v is off every face (no ghost
 * vertex, no table); the kernel axes of the mesh are [3 - D, 3). */
template <bool SMEM, typename T>
__device__ __forceinline__ T ld_(const T* a) {
  if constexpr (SMEM) return *a;
  else return __ldcg(a);
}

template <typename T, int CS, int D, bool EDGE, bool SMEM = false>
__device__ __forceinline__ T estimate(const Geo<T>& g, const T* __restrict__ cur, const T* __restrict__ coef, T lap,
                                      int c, int z, int i, int j, int v) {
  constexpr int FIRST = 3 - D;
  const int q[3] = {z, i, j};
  const int ir = q[FIRST];  // index along mesh axis 0 (r for curvilinear meshes)
  T acc = T(0);
#pragma unroll
  for (int ka = FIRST; ka < 3; ++ka) {
    const int a = ka - FIRST;  // mesh axis
    const int s = g.stride[ka];
    T prev, next;
    if (!EDGE || q[ka] > 0) {
      prev = ld_<SMEM>(cur + v - s);
    } else {
      T gv;
      prev = table_value(g, g.neu, g.nmask, 2 * ka, c, z, i, j, gv) ? add_(ld_<SMEM>(cur + v + s), mul_(-g.two_dx[ka], gv))
                                                                    : T(0);
    }
    if (!EDGE || q[ka] < g.n[ka] - 1) {
      next = ld_<SMEM>(cur + v + s);
    } else {
      T gv;
      next = table_value(g, g.neu, g.nmask, 2 * ka + 1, c, z, i, j, gv) ? add_(ld_<SMEM>(cur + v - s), mul_(g.two_dx[ka], gv))
                                                                       : T(0);
    }
    const T upd = mul_(add_(prev, next), g.inv_dxx[ka]);
    T term = upd;
    if (CS == 1 || CS == 2) {  // polar / cylindrical: r along mesh axis 0
      const int nr = g.n[FIRST];
      if (a == 0) term = add_(upd, mul_(sub_(next, prev), coef[ir]));
      else if (a == 1) term = mul_(upd, coef[nr + ir]);
    } else if (CS == 3) {  // spherical: r along axis 0, phi along axis 2
      const int nr = g.n[0], np = g.n[2];
      if (a == 0) term = add_(upd, mul_(sub_(next, prev), coef[z]));
      else if (a == 1) term = mul_(upd, coef[2 * nr + 2 * np + z * np + j]);
      else term = mul_(add_(upd, mul_(mul_(coef[2 * nr + j], sub_(next, prev)), coef[2 * nr + np + j])), coef[nr + z]);
    }
    acc = (a == 0) ? term : add_(acc, term);
  }
  acc = sub_(acc, lap);
  T inv_den;
  if (CS == 0) inv_den = coef[0];
  else if (CS == 1 || CS == 2) inv_den = coef[2 * g.n[FIRST] + ir];
  else inv_den = coef[2 * g.n[0] + 2 * g.n[2] + g.n[0] * g.n[2] + z * g.n[2] + j];
  return mul_(acc, inv_den);
}

/* Dirichlet values in face order (later axes win at edges and corners). */
template <typename T, int D>
__device__ __forceinline__ T constrain(const Geo<T>& g, T v, int c, int z, int i, int j) {
#pragma unroll
  for (int f = 2 * (3 - D); f < 6; ++f) {
    const int ka = f >> 1;
    const int q = ka == 0 ? z : (ka == 1 ? i : j);
    if (q != ((f & 1) ? g.n[ka] - 1 : 0)) continue;
    T d;
    if (table_value(g, g.dir, g.dmask, f, c, z, i, j, d)) v = d;
  }
  return v;
}

template <int D>
__device__ __forceinline__ void decode(int v, const Div& d12, const Div& d2, int& z, int& i, int& j) {
  if (D == 3) {
    z = div_(v, d12);
    const int r = v - z * d12.d;
    i = div_(r, d2);
    j = r - i * d2.d;
  } else if (D == 2) {
    z = 0;
    i = div_(v, d2);
    j = v - i * d2.d;
  } else {
    z = 0;
    i = 0;
    j = v;
  }
}

template <typename T, int CS, int D>
__global__ void __launch_bounds__(JT) jacobi_kernel(const prml_jacobi_params p, T* __restrict__ state,
                                                   const double* __restrict__ y_init, unsigned char* scratch,
                                                   Layout L, int G, Div d12, Div d2) {
  constexpr int FIRST = 3 - D;
  __shared__ double red[JT / 32];
  __shared__ unsigned char done[PRML_JACOBI_MAX_BATCH];
  __shared__ int final_buf[PRML_JACOBI_MAX_BATCH];
  __shared__ int lapc[16];
  __shared__ int stop;

  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(scratch + L.control);
  unsigned* status = reinterpret_cast<unsigned*>(scratch + L.control + 128);
  long long* iters = reinterpret_cast<long long*>(scratch + L.iters);
  double* partial = reinterpret_cast<double*>(scratch + L.partial);
  T* const buf0 = reinterpret_cast<T*>(scratch + L.buf0);
  T* const buf1 = reinterpret_cast<T*>(scratch + L.buf1);
  const T* coef = static_cast<const T*>(p.coef);
  const int n_lap = p.n_lap, batch = p.batch;
  const double tol = p.tol;

  Geo<T> g;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    g.n[a] = p.n[a];
    g.inv_dxx[a] = T(p.inv_dxx[a]);
    g.two_dx[a] = T(p.two_dx[a]);
  }
  g.V = g.n[0] * g.n[1] * g.n[2];
  g.stride[2] = 1;
  g.stride[1] = g.n[2];
  g.stride[0] = g.n[1] * g.n[2];
  g.d12 = d12;
  g.d2 = d2;
  g.dir = static_cast<const T*>(p.dirichlet);
  g.neu = static_cast<const T*>(p.neumann);
  g.dmask = p.dir_mask;
  g.nmask = p.neu_mask;
  g.comps = p.comps;
  g.flen = p.face_len;
  g.fbase = p.face_base;
  g.pitch = p.pitch;
  g.cstride = p.cstride;

  const int b = blockIdx.x / G;      // instance of this CTA
  const int k = blockIdx.x - b * G;  // CTA index within the instance
  /* this CTA's vertices [v0, v1) of its instance, every solved component */
  const int per = (g.V + G - 1) / G;
  const int v0 = k * per, v1 = min(g.V, v0 + per);
  T* st = state + (long long)b * p.inst;
  const long long ib = (long long)b * n_lap * g.V;
  unsigned long long target = 0;

  if (threadIdx.x < 16) lapc[threadIdx.x] = p.lap_comp[threadIdx.x];
  for (int bb = threadIdx.x; bb < batch; bb += JT) {
    done[bb] = 0;
    final_buf[bb] = 0;
  }
  __syncthreads();

  /* constrained initial estimate into buffer 0 */
  for (int v = v0 + threadIdx.x; v < v1; v += JT) {
    int z, i, j;
    decode<D>(v, d12, d2, z, i, j);
    for (int l = 0; l < n_lap; ++l) {
      const T y0 = T(y_init[((long long)b * g.V + v) * n_lap + l]);
      __stcg(buf0 + ib + (long long)l * g.V + v, constrain<T, D>(g, y0, lapc[l], z, i, j));
    }
  }
  grid_sync(cnt, status, target);

  /* the reference's loop starts from an infinite change: tol = inf runs no
   * iteration and returns the constrained initial estimate */
  long long it = -1;
  if (!(__longlong_as_double(0x7ff0000000000000LL) > tol)) {
    for (int bb = threadIdx.x; bb < batch; bb += JT) done[bb] = 1;
    if (k == 0 && threadIdx.x == 0) iters[b] = 0;
    __syncthreads();
  } else for (it = 0;; ++it) {
    const T* __restrict__ cur = ((it & 1) ? buf1 : buf0) + ib;
    T* __restrict__ nxt = ((it & 1) ? buf0 : buf1) + ib;
    T sq = T(0);
    if (!done[b]) {
      for (int v = v0 + threadIdx.x; v < v1; v += JT) {
        int z, i, j;
        decode<D>(v, d12, d2, z, i, j);
        bool interior = j > 0 && j < g.n[2] - 1;
        if (FIRST <= 1) interior = interior && i > 0 && i < g.n[1] - 1;
        if (FIRST == 0) interior = interior && z > 0 && z < g.n[0] - 1;
        const long long so = ((long long)z * g.n[1] + i) * g.pitch + j;
        for (int l = 0; l < n_lap; ++l) {
          const int c = lapc[l];
          const T* cl = cur + (long long)l * g.V;
          const T lap = st[c * g.cstride + so];
          const T old = __ldcg(cl + v);
          T y;
          if (interior) {
            y = estimate<T, CS, D, false>(g, cl, coef, lap, c, z, i, j, v);
          } else {
            y = estimate<T, CS, D, true>(g, cl, coef, lap, c, z, i, j, v);
            y = constrain<T, D>(g, y, c, z, i, j);
          }
          __stcg(nxt + (long long)l * g.V + v, y);
          const T d = y - old;
          sq = fma_(d, d, sq);
        }
      }
    }
    const double s = block_sum<JT, T>(sq, reinterpret_cast<T*>(red));
    if (threadIdx.x == 0) partial[((it & 1) * batch + b) * G + k] = s;
    grid_sync(cnt, status, target);
    /* warp 0 of every CTA evaluates every instance's norm in the same order */
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      int all = 1;
      for (int bb = 0; bb < batch; ++bb) {
        if (done[bb]) continue;
        double t = 0.0;
        for (int kk = lane; kk < G; kk += 32) t += __ldcg(partial + ((it & 1) * batch + bb) * G + kk);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (!(sqrt(t) > tol)) {
          if (lane == 0) {
            done[bb] = 1;
            final_buf[bb] = (int)((it + 1) & 1);
            if (k == 0 && bb == b) iters[bb] = it + 1;
          }
        } else {
          all = 0;
        }
      }
      if (lane == 0) {
        const bool capped = it + 1 >= p.max_iterations;
        const bool failed = (ld_acquire32(status) & 2u) != 0;
        stop = all || capped || failed;
      }
    }
    __syncthreads();
    if (stop) break;
  }

  if (!done[b]) {
    if (k == 0 && threadIdx.x == 0) iters[b] = -1;
    if (threadIdx.x == 0) final_buf[b] = (int)((it + 1) & 1);  // the latest estimate
    __syncthreads();
  }
  /* result into the solved components' planes of the state */
  const T* fin = (final_buf[b] ? buf1 : buf0) + ib;
  for (int v = v0 + threadIdx.x; v < v1; v += JT) {
    int z, i, j;
    decode<D>(v, d12, d2, z, i, j);
    const long long so = ((long long)z * g.n[1] + i) * g.pitch + j;
    for (int l = 0; l < n_lap; ++l) st[lapc[l] * g.cstride + so] = __ldcg(fin + (long long)l * g.V + v);
  }
}

/* Staged kernel: CTA k of an instance owns the units [r0, r1) of the
 * outermost kernel axis of the mesh (planes of a 3D mesh, rows otherwise; a
 * 1D mesh is one row) and keeps units [r0 - K, r1 + K) of the estimates and
 * of the right-hand side in shared memory.  One block = K Jacobi iterations
 * on chip: iteration s computes every staged unit whose neighbours are
 * still valid (the band shrinks by one unit per side and iteration, except
 * at the mesh faces), so after K iterations the owned units hold exactly the
 * values of K global iterations; each iteration's squared change over the
 * owned units goes to `partial`, the owned units go to global memory, and
 * one grid barrier ends the block.  Every CTA then finds, in the same
 * order, the first iteration of the block at or below tol.  An instance that
 * stopped inside a block (or hit the iteration cap) is finished by
 * re-running that block from its start up to the stop iteration, which
 * reproduces the same values, and storing the owned units. */
template <typename T>
struct Stage {
  int unit;      // vertices per unit
  int nu;        // units of the mesh
  int per;       // units owned per CTA
  int K;         // iterations per block
  int R;         // staged units (per + 2K, clipped to the mesh)
  Div dn2;       // division by the line length n2
  Div dl;        // division by the lines of a unit (3D: n1)
};

/* Runs `steps` iterations of the block on the staged estimates in sA;
 * returns the buffer holding the result.  The computable vertices (lines of
 * n2 contiguous vertices; a unit is one line, or n1 lines of a 3D plane)
 * are split evenly over the CTA's threads, indexes decoded by multiply and
 * shift.  Thread 0 stores each iteration's owned squared change in part[s]
 * when part is not null. */
template <typename T, int CS, int D>
__device__ __forceinline__ T* run_block(const Geo<T>& g, const Stage<T>& sg, const T* coef, const int* lapc, int n_lap,
                                        T* sA, T* sB, const T* sR, int sr0, int sr1, int r0, int r1, int steps,
                                        double* part, double* red2) {
  using Acc = T;
  const int R = sr1 - sr0;
  const int n2 = g.n[2];
  const int lpu = D == 3 ? g.n[1] : 1;  // lines per unit
  int vlo = sr0, vhi = sr1;
  T* src = sA;
  T* dst = sB;
  for (int s = 0; s < steps; ++s) {
    const int nlo = (sr0 == 0) ? 0 : vlo + 1;
    const int nhi = (sr1 == sg.nu) ? sg.nu : vhi - 1;
    Acc sq = Acc(0);
    const int count = (nhi - nlo) * lpu * n2;
    for (int idx = threadIdx.x; idx < count; idx += JS) {
      const int line = div_(idx, sg.dn2);
      const int j = idx - line * n2;
      const int du = D == 3 ? div_(line, sg.dl) : line;
      const int gu = nlo + du;
      const int z = D == 3 ? gu : 0;
      const int i = D == 3 ? line - du * lpu : (D == 2 ? gu : 0);
      bool in = j > 0 && j < n2 - 1;  // off every face
      if (D >= 2) in = in && i > 0 && i < g.n[1] - 1;
      if (D == 3) in = in && z > 0 && z < g.n[0] - 1;
      const bool own = gu >= r0 && gu < r1;
      const int v = gu * sg.unit + (D == 3 ? i * n2 : 0) + j;
      for (int l = 0; l < n_lap; ++l) {
        const int c = lapc[l];
        const int lo = (l * R - sr0) * sg.unit;  // local index of dense vertex v is v + lo
        const T* cl = src + lo;
        const T old = cl[v];
        T y;
        if (in) {
          y = estimate<T, CS, D, false, true>(g, cl, coef, sR[v + lo], c, z, i, j, v);
        } else {
          y = estimate<T, CS, D, true, true>(g, cl, coef, sR[v + lo], c, z, i, j, v);
          y = constrain<T, D>(g, y, c, z, i, j);
        }
        dst[v + lo] = y;
        if (own) {
          const Acc d = Acc(y) - Acc(old);
          sq = fma_(d, d, sq);
        }
      }
    }
    /* one CTA barrier per iteration: it also completes dst for the next */
    const double tot = block_sum<JS, Acc>(sq, reinterpret_cast<Acc*>(red2 + (s & 1) * (JS / 32)));
    if (part && threadIdx.x == 0) part[s] = tot;
    T* t = src;
    src = dst;
    dst = t;
    vlo = nlo;
    vhi = nhi;
  }
  __syncthreads();
  return src;
}

template <typename T, int CS, int D>
__global__ void __launch_bounds__(JS) jacobi_staged(const prml_jacobi_params p, T* __restrict__ state,
                                                   const double* __restrict__ y_init, unsigned char* scratch,
                                                   Layout L, int G, Div d12, Div d2, Stage<T> sg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red2[2 * (JS / 32)];
  __shared__ int dec_s[PRML_JACOBI_MAX_BATCH];
  __shared__ double kpart[8];
  __shared__ unsigned char done[PRML_JACOBI_MAX_BATCH];
  __shared__ unsigned char fin_par[PRML_JACOBI_MAX_BATCH];
  __shared__ unsigned char fin_steps[PRML_JACOBI_MAX_BATCH];
  __shared__ int lapc[16];
  __shared__ int stop;

  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(scratch + L.control);
  unsigned* status = reinterpret_cast<unsigned*>(scratch + L.control + 128);
  unsigned long long* release = reinterpret_cast<unsigned long long*>(scratch + L.control + 64);
  int* dec = reinterpret_cast<int*>(scratch + L.dec);
  long long* iters = reinterpret_cast<long long*>(scratch + L.iters);
  double* partial = reinterpret_cast<double*>(scratch + L.partial);
  T* const buf0 = reinterpret_cast<T*>(scratch + L.buf0);
  T* const buf1 = reinterpret_cast<T*>(scratch + L.buf1);
  const T* coef = static_cast<const T*>(p.coef);
  const int n_lap = p.n_lap, batch = p.batch;
  const double tol = p.tol;

  Geo<T> g;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    g.n[a] = p.n[a];
    g.inv_dxx[a] = T(p.inv_dxx[a]);
    g.two_dx[a] = T(p.two_dx[a]);
  }
  g.V = g.n[0] * g.n[1] * g.n[2];
  g.stride[2] = 1;
  g.stride[1] = g.n[2];
  g.stride[0] = g.n[1] * g.n[2];
  g.d12 = d12;
  g.d2 = d2;
  g.dir = static_cast<const T*>(p.dirichlet);
  g.neu = static_cast<const T*>(p.neumann);
  g.dmask = p.dir_mask;
  g.nmask = p.neu_mask;
  g.comps = p.comps;
  g.flen = p.face_len;
  g.fbase = p.face_base;
  g.pitch = p.pitch;
  g.cstride = p.cstride;

  const int b = blockIdx.x / G;
  const int k = blockIdx.x - b * G;
  const int r0 = min(sg.nu, k * sg.per), r1 = min(sg.nu, r0 + sg.per);
  const int sr0 = max(0, r0 - sg.K), sr1 = min(sg.nu, r1 + sg.K);
  const int R = sr1 - sr0;
  const int unit = sg.unit;
  T* sA = reinterpret_cast<T*>(smem_raw);
  T* sB = sA + (size_t)n_lap * sg.R * unit;
  T* sR = sB + (size_t)n_lap * sg.R * unit;
  T* st = state + (long long)b * p.inst;
  const long long ib = (long long)b * n_lap * g.V;
  unsigned long long target = 0;

  if (threadIdx.x < 16) lapc[threadIdx.x] = p.lap_comp[threadIdx.x];
  for (int bb = threadIdx.x; bb < batch; bb += JS) {
    done[bb] = 0;
    fin_par[bb] = 0;
    fin_steps[bb] = 0;
  }
  __syncthreads();

  /* constrained initial estimate of the owned units into buffer 0, and the
   * right-hand side of the staged units into shared memory */
  for (int idx = threadIdx.x; idx < (r1 - r0) * unit; idx += JS) {
    const int v = r0 * unit + idx;
    int z, i, j;
    decode<D>(v, d12, d2, z, i, j);
    for (int l = 0; l < n_lap; ++l) {
      const T y0 = T(y_init[((long long)b * g.V + v) * n_lap + l]);
      __stcg(buf0 + ib + (long long)l * g.V + v, constrain<T, D>(g, y0, lapc[l], z, i, j));
    }
  }
  for (int idx = threadIdx.x; idx < R * unit; idx += JS) {
    const int v = sr0 * unit + idx;
    int z, i, j;
    decode<D>(v, d12, d2, z, i, j);
    const long long so = ((long long)z * g.n[1] + i) * g.pitch + j;
    for (int l = 0; l < n_lap; ++l) sR[(l * R) * unit + idx] = st[lapc[l] * g.cstride + so];
  }
  grid_sync(cnt, status, target);

  long long it0 = 0;
  int par = 0;  // the block's start estimates are in buffer `par`
  if (!(__longlong_as_double(0x7ff0000000000000LL) > tol)) {
    /* tol = inf: no iteration, the constrained initial estimate */
    for (int bb = threadIdx.x; bb < batch; bb += JS) done[bb] = 1;
    if (k == 0 && threadIdx.x == 0) iters[b] = 0;
    __syncthreads();
  } else {
    for (;;) {
      const long long left = p.max_iterations - it0;
      const int Kb = (int)(left < sg.K ? left : sg.K);
      const T* cur = (par ? buf1 : buf0) + ib;
      T* nxt = (par ? buf0 : buf1) + ib;
      if (!done[b]) {
        for (int l = 0; l < n_lap; ++l) {
          const T* gsrc = cur + (long long)l * g.V + (long long)sr0 * unit;
          T* sdst = sA + (size_t)l * R * unit;
          for (int idx = threadIdx.x; idx < R * unit; idx += JS) sdst[idx] = __ldcg(gsrc + idx);
        }
        __syncthreads();
        T* fin = run_block<T, CS, D>(g, sg, coef, lapc, n_lap, sA, sB, sR, sr0, sr1, r0, r1, Kb, kpart, red2);
        for (int l = 0; l < n_lap; ++l) {
          const T* ssrc = fin + (size_t)l * R * unit + (size_t)(r0 - sr0) * unit;
          T* gdst = nxt + (long long)l * g.V + (long long)r0 * unit;
          for (int idx = threadIdx.x; idx < (r1 - r0) * unit; idx += JS) __stcg(gdst + idx, ssrc[idx]);
        }
      } else if (threadIdx.x < 8) {
        kpart[threadIdx.x] = 0.0;
      }
      if (threadIdx.x < Kb) partial[(((long long)par * 8 + threadIdx.x) * batch + b) * G + k] = kpart[threadIdx.x];
      /* Barrier and stop decision in one: the last CTA to arrive reads every
       * CTA's partial norms, decides for every instance (first iteration of
       * the block at or below tol) and publishes the decisions with the
       * release; the others wait for the release and read them.  Waits are
       * bounded like grid_sync's. */
      __syncthreads();
      target += gridDim.x;
      if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int last = 0;
        if (lane == 0) {
          __threadfence();
          last = atomicAdd(cnt, 1ull) + 1 == target;
          __threadfence();
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (last) {
          int all = 1;
          for (int bb = 0; bb < batch; ++bb) {
            if (done[bb]) continue;
            double t[8];
#pragma unroll
            for (int s = 0; s < 8; ++s) t[s] = 0.0;
#pragma unroll 4
            for (int kk = lane; kk < G; kk += 32) {
#pragma unroll
              for (int s = 0; s < 8; ++s)
                if (s < Kb) t[s] += __ldcg(partial + (((long long)par * 8 + s) * batch + bb) * G + kk);
            }
            int hit = -1;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
#pragma unroll
              for (int o = 16; o > 0; o >>= 1) t[s] += __shfl_xor_sync(0xffffffffu, t[s], o);
              if (hit < 0 && s < Kb && !(sqrt(t[s]) > tol)) hit = s;
            }
            if (lane == 0) __stcg(dec + bb, hit);
            all &= hit >= 0;
          }
          if (lane == 0) {
            const bool capped = it0 + Kb >= p.max_iterations;
            const bool failed = (ld_acquire32(status) & 2u) != 0;
            const int stop_now = all || capped || failed;
            __threadfence();
            asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(release), "l"(target * 2 + stop_now) : "memory");
            stop = stop_now;
          }
        } else {
          if (lane == 0) {
            const unsigned long long t0 = global_ns();
            unsigned long long r = ld_acquire64(release);
            while ((r >> 1) < target) {
              __nanosleep(32);
              if (global_ns() - t0 > BARRIER_NS) {
                atomicOr(status, 2u);
                r = 1;  // stop
                break;
              }
              r = ld_acquire64(release);
            }
            stop = (int)(r & 1ull);
          }
        }
        __syncwarp();
        /* apply the decisions (identical in every CTA) */
        for (int bb = lane; bb < batch; bb += 32) dec_s[bb] = done[bb] ? -2 : __ldcg(dec + bb);
        __syncwarp();
        if (lane == 0) {
          const bool capped = it0 + Kb >= p.max_iterations;
          for (int bb = 0; bb < batch; ++bb) {
            if (done[bb]) continue;
            const int hit = dec_s[bb];
            if (hit >= 0) {
              done[bb] = 1;
              fin_par[bb] = (unsigned char)par;
              fin_steps[bb] = (unsigned char)(hit + 1);
              if (k == 0 && bb == b) iters[bb] = it0 + hit + 1;
            } else if (capped) {
              fin_par[bb] = (unsigned char)par;  // the latest estimate: the whole block
              fin_steps[bb] = (unsigned char)Kb;
              if (k == 0 && bb == b) iters[bb] = -1;
            }
          }
        }
      }
      __syncthreads();
      it0 += Kb;
      par ^= 1;
      if (stop) break;
    }
  }

  /* the result: re-run the stop block from its start up to the stop
   * iteration (no iteration for tol = inf) and store the owned units */
  const int steps = fin_steps[b];
  const T* cur = (fin_par[b] ? buf1 : buf0) + ib;
  for (int l = 0; l < n_lap; ++l) {
    const T* gsrc = cur + (long long)l * g.V + (long long)sr0 * unit;
    T* sdst = sA + (size_t)l * R * unit;
    for (int idx = threadIdx.x; idx < R * unit; idx += JS) sdst[idx] = __ldcg(gsrc + idx);
  }
  __syncthreads();
  const T* fin = run_block<T, CS, D>(g, sg, coef, lapc, n_lap, sA, sB, sR, sr0, sr1, r0, r1, steps, nullptr, red2);
  for (int idx = threadIdx.x; idx < (r1 - r0) * unit; idx += JS) {
    const int v = r0 * unit + idx;
    int z, i, j;
    decode<D>(v, d12, d2, z, i, j);
    const long long so = ((long long)z * g.n[1] + i) * g.pitch + j;
    for (int l = 0; l < n_lap; ++l)
      st[lapc[l] * g.cstride + so] = fin[(size_t)l * R * unit + (size_t)(r0 - sr0) * unit + idx];
  }
}

constexpr int STAGED_SMEM_MAX = 200 * 1024;

/* Launch shape of the staged kernel.  A CTA owning `per` units with K
 * iterations per block computes per + K - 1 units per iteration, so the
 * redundant work is (K - 1) / per, against one grid barrier per K
 * iterations.  float64 (FP64 issue rate is the limit on this GPU): K = 4 and
 * one unit per CTA, spreading the work over as many SMs as there are units;
 * float32: K = 8 and two units per CTA.  Both own at least JS / 2 vertices
 * per CTA; per grows until all CTAs are co-resident; K halves if the band
 * does not fit in shared memory.  False: use the direct kernel. */
template <typename T, int CS, int D>
bool staged_shape(const prml_jacobi_params& p, int sms, Stage<T>& sg, int& G, int& smem) {
  const int unit = D == 3 ? p.n[1] * p.n[2] : p.n[2];
  const int nu = D == 3 ? p.n[0] : p.n[1];
  const int esize = (int)sizeof(T);
  for (int K = sizeof(T) == 8 ? 4 : 8; K >= 1; K >>= 1) {
    int per = sizeof(T) == 8 ? 1 : 2;
    if (per * unit < JS / 2) per = (JS / 2 + unit - 1) / unit;  // at least JS / 2 owned vertices
    for (int guard = 0; guard < 64; ++guard) {
      const int g = (nu + per - 1) / per;
      const int R = per + 2 * K < nu ? per + 2 * K : nu;
      const long long bytes = 3LL * p.n_lap * R * unit * esize;
      if (bytes > STAGED_SMEM_MAX) break;
      auto kern = jacobi_staged<T, CS, D>;
      if (cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
        return false;
      int occ = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, JS, (size_t)bytes);
      if (occ < 1) break;
      const int cap = occ * sms / p.batch;
      if (cap >= 1 && g <= cap) {
        sg.unit = unit;
        sg.nu = nu;
        sg.per = per;
        sg.K = K;
        sg.R = R;
        sg.dn2 = make_div(p.n[2]);
        sg.dl = make_div(D == 3 ? p.n[1] : 1);
        G = g;
        smem = (int)bytes;
        return true;
      }
      const int want = cap >= 1 ? (nu + cap - 1) / cap : 2 * per;
      per = want > per ? want : per + 1;
    }
  }
  return false;
}

template <typename T, int CS, int D>
int launch(const prml_jacobi_params& p, void* state, const double* y_init, void* scratch, long long scratch_bytes,
           long long* iterations, cudaStream_t s) {
  int dev = 0, sms = 0, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!coop) return prml_set_error(PRML_ERR_CUDA, "prml_anti_laplacian: cooperative launch unavailable");
  const long long V = (long long)p.n[0] * p.n[1] * p.n[2];
  Stage<T> sg{};
  int G = 0, smem = 0;
  const bool staged = staged_shape<T, CS, D>(p, sms, sg, G, smem);
  const void* kern;
  if (staged) {
    kern = (const void*)jacobi_staged<T, CS, D>;
  } else {
    int occ = 0;
    kern = (const void*)jacobi_kernel<T, CS, D>;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, jacobi_kernel<T, CS, D>, JT, 0);
    if (occ < 1) return prml_set_error(PRML_ERR_CUDA, "prml_anti_laplacian: kernel does not fit on an SM");
    /* about two vertices per thread (latency-bound loads), as far as the
     * co-resident CTAs allow */
    long long g = (V + 2 * JT - 1) / (2 * JT);
    const long long cap = (long long)occ * sms / p.batch;
    if (g > cap) g = cap;
    if (g < 1) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: batch exceeds co-resident CTAs");
    G = (int)g;
  }
  const Layout L = layout_of(p, G);
  if (scratch_bytes < L.total) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: scratch too small");
  cudaError_t e = cudaMemsetAsync(scratch, 0, 256, s);
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("prml_anti_laplacian: ") + cudaGetErrorString(e));
  T* st = static_cast<T*>(state);
  unsigned char* sc = static_cast<unsigned char*>(scratch);
  prml_jacobi_params pc = p;
  Layout Lc = L;
  Div d12 = make_div(p.n[1] * p.n[2]), d2 = make_div(p.n[2]);
  void* args_direct[] = {&pc, &st, (void*)&y_init, &sc, &Lc, &G, &d12, &d2};
  void* args_staged[] = {&pc, &st, (void*)&y_init, &sc, &Lc, &G, &d12, &d2, &sg};
  e = cudaLaunchCooperativeKernel(kern, dim3((unsigned)(G * p.batch)), dim3(staged ? JS : JT), staged ? args_staged : args_direct,
                                  staged ? (size_t)smem : 0, s);
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("prml_anti_laplacian launch: ") + cudaGetErrorString(e));
  long long its[PRML_JACOBI_MAX_BATCH];
  unsigned ctl[4];
  cudaMemcpyAsync(its, sc + L.iters, 8LL * p.batch, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(ctl, sc + 128, 16, cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("prml_anti_laplacian: ") + cudaGetErrorString(e));
  if (ctl[0] & 2u) return prml_set_error(PRML_ERR_CUDA, "prml_anti_laplacian: grid barrier timed out");
  if (iterations)
    for (int b = 0; b < p.batch; ++b) iterations[b] = its[b];
  for (int b = 0; b < p.batch; ++b)
    if (its[b] < 0)
      return prml_set_error(PRML_ERR_CONVERGENCE, "prml_anti_laplacian: no convergence within max_iterations (instance " +
                                                      std::to_string(b) + ")");
  return PRML_OK;
}

int check(const prml_jacobi_params* p) {
  if (!p) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: null parameters");
  if (p->elem_bytes != 4 && p->elem_bytes != 8) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: elem_bytes must be 4 or 8");
  if (p->batch < 1 || p->batch > PRML_JACOBI_MAX_BATCH)
    return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: batch must be 1.." + std::to_string(PRML_JACOBI_MAX_BATCH));
  if (p->n_lap < 1 || p->n_lap > 16 || p->comps < p->n_lap || p->comps > 16)
    return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: bad component counts");
  if (p->first_axis < 0 || p->first_axis > 2) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: bad first_axis");
  for (int a = 0; a < 3; ++a) {
    if (p->n[a] < 1) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: bad mesh extent");
    /* numerical_differentiator.py:1103-1106 */
    if (a >= p->first_axis && p->n[a] < 3)
      return prml_set_error(PRML_ERR_ARG, "y must contain at least 3 points along all x axes");
    if (a < p->first_axis && p->n[a] != 1) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: bad mesh extent");
  }
  if ((long long)p->n[0] * p->n[1] * p->n[2] >= (1LL << 31))
    return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: more than 2^31 vertices per instance");
  for (int l = 0; l < p->n_lap; ++l)
    if (p->lap_comp[l] < 0 || p->lap_comp[l] >= p->comps) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: bad component");
  if (p->coord_system < 0 || p->coord_system > 3) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: bad coordinate system");
  if (p->coord_system == 3 && p->first_axis != 0)
    return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: spherical meshes are 3D");
  if (p->coord_system == 2 && p->first_axis != 0)
    return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: cylindrical meshes are 3D");
  if (p->coord_system == 1 && p->first_axis != 1)
    return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: polar meshes are 2D");
  if (!p->coef || !p->dirichlet || !p->neumann) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: null table");
  /* numerical_differentiator.py:26-27: only a negative tolerance is refused */
  if (p->max_iterations < 1 || p->tol < 0.0) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: bad tol or max_iterations");
  return PRML_OK;
}

}  // namespace

extern "C" {

int prml_jacobi_params_size(void) { return (int)sizeof(prml_jacobi_params); }

long long prml_jacobi_scratch_bytes(const prml_jacobi_params* p) {
  if (check(p) != PRML_OK) return -1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1024;
  /* upper bound on G: every SM full of CTAs of JT threads */
  const int G = sms * (2048 / JT);
  return layout_of(*p, G).total;
}

int prml_anti_laplacian(const prml_jacobi_params* p, void* state, const double* y_init, void* scratch,
                        long long scratch_bytes, long long* iterations, void* stream) {
  int rc = check(p);
  if (rc != PRML_OK) return rc;
  if (!state || !y_init || !scratch) return prml_set_error(PRML_ERR_ARG, "prml_anti_laplacian: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int cs = p->coord_system, d = 3 - p->first_axis;
#define PRML_JACOBI_CASES(T)                                                                   \
  if (cs == 0 && d == 1) return launch<T, 0, 1>(*p, state, y_init, scratch, scratch_bytes, iterations, s); \
  if (cs == 0 && d == 2) return launch<T, 0, 2>(*p, state, y_init, scratch, scratch_bytes, iterations, s); \
  if (cs == 0 && d == 3) return launch<T, 0, 3>(*p, state, y_init, scratch, scratch_bytes, iterations, s); \
  if (cs == 1) return launch<T, 1, 2>(*p, state, y_init, scratch, scratch_bytes, iterations, s);           \
  if (cs == 2) return launch<T, 2, 3>(*p, state, y_init, scratch, scratch_bytes, iterations, s);           \
  return launch<T, 3, 3>(*p, state, y_init, scratch, scratch_bytes, iterations, s);
  if (p->elem_bytes == 8) {
    PRML_JACOBI_CASES(double)
  }
  PRML_JACOBI_CASES(float)
#undef PRML_JACOBI_CASES
}

}  // extern "C"
