/*
 * Fused finite-difference step kernel (one launch = one full integrator step).
 *
 * Compiled at run time by NVRTC together with a generated equation struct
 * `Eq` (see pararealml_gb300/codegen.py).  One CTA owns a TX x TY tile of
 * output vertices of one instance.  It stages the tile plus a halo (rows:
 * one vertex per stage; columns: the same rounded up to a 16-byte boundary)
 * of every component of the input state in shared memory with a single TMA
 * box load, then evaluates the integrator's stages in shared memory on
 * shrinking regions (tile + NSTAGE-1-s for stage s), so that every stage
 * input is produced on-chip and only the final state goes back to global
 * memory.  Per step the state is read once (plus halo) and written once.
 *
 * Semantics reproduced from the reference (ViktorC/PararealML):
 *   - ThreePointCentralDifferenceMethod._derivative
 *     (operators/fdm/numerical_differentiator.py:1012-1057): zero halo
 *     outside the domain, then a Neumann value, where one is given,
 *     overwrites the boundary derivative.
 *   - _second_derivative + _add_halos_along_axis (:1059-1095, :1188-1242):
 *     ghost vertices y[1] - 2dx*g (lower) and y[n-2] + 2dx*g (upper) where a
 *     Neumann value is given, zero otherwise; mixed second derivatives are
 *     the unconstrained derivative of the constrained derivative.
 *   - ForwardEulerMethod / ExplicitMidpointMethod / RK4
 *     (operators/fdm/numerical_integrator.py:42-132): Dirichlet values are
 *     re-imposed on every stage input and on the result.
 *   - FDMOperator._create_y_next_function (operators/fdm/fdm_operator.py:
 *     79-165): components whose left-hand side is not dy/dt get dy/dt = 0
 *     inside the stages; LHS.Y components are set, after the step, to their
 *     right-hand side evaluated at (t, y_old) and then constrained.
 *   - constrained_problem.py:262-301: Dirichlet faces are applied in axis
 *     order, lower then upper, so later axes win at corners.
 *
 * Face numbering: 0/1 = lower/upper face of kernel axis 0 (rows i = 0 and
 * i = nx-1, indexed by column j), 2/3 = lower/upper face of kernel axis 1
 * (cols j = 0 and j = ny-1, indexed by row i).  Tables hold NaN where a
 * vertex is unconstrained.
 */
#pragma once
#include "prml_params.h"

namespace prml {

enum Integrator { FORWARD_EULER = 1, EXPLICIT_MIDPOINT = 2, RK4 = 4 };

template <typename T>
struct MeshC {
  T inv2d0, inv2d1, invdd0, invdd1, twod0, twod1;
  int nx, ny, flen;
  const T* dir;
  const T* neu;
  const double* c0;
  const double* c1;
};

/* A vertex of the current stage input, with the stencil operators the
 * generated right-hand sides call. */
template <typename T, class Eq, int RY, int RXY>
struct Point {
  using real = T;
  const T* s;
  int l;
  int gi, gj;
  const MeshC<T>* m;
  double time;

  __device__ __forceinline__ T v(int c, int di, int dj) const {
    return s[c * RXY + l + di * RY + dj];
  }
  __device__ __forceinline__ T face(const T* tab, int f, int c, int k) const {
    return tab[(f * Eq::C + c) * m->flen + k];
  }
  static __device__ __forceinline__ constexpr bool has_neu(int f, int c) {
    return (Eq::NEU_MASK >> (f * Eq::C + c)) & 1ull;
  }

  template <int c> __device__ __forceinline__ T val() const { return v(c, 0, 0); }
  __device__ __forceinline__ T t() const { return T(time); }
  template <int ka> __device__ __forceinline__ T x() const {
    return ka == 0 ? T(m->c0[gi]) : T(m->c1[gj]);
  }

  /* Constrained first derivative along kernel axis ka at the vertex offset
   * by (di, dj); zero outside the domain when CHECK is set. */
  template <int c, int ka, bool CHECK>
  __device__ __forceinline__ T grad_at(int di, int dj) const {
    const int qi = gi + di, qj = gj + dj;
    if (CHECK && (qi < 0 || qi >= m->nx || qj < 0 || qj >= m->ny)) return T(0);
    if (ka == 0) {
      if (has_neu(0, c) && qi == 0) {
        const T g = face(m->neu, 0, c, qj);
        if (g == g) return g;
      }
      if (has_neu(1, c) && qi == m->nx - 1) {
        const T g = face(m->neu, 1, c, qj);
        if (g == g) return g;
      }
      return (v(c, di + 1, dj) - v(c, di - 1, dj)) * m->inv2d0;
    } else {
      if (has_neu(2, c) && qj == 0) {
        const T g = face(m->neu, 2, c, qi);
        if (g == g) return g;
      }
      if (has_neu(3, c) && qj == m->ny - 1) {
        const T g = face(m->neu, 3, c, qi);
        if (g == g) return g;
      }
      return (v(c, di, dj + 1) - v(c, di, dj - 1)) * m->inv2d1;
    }
  }
  template <int c, int ka> __device__ __forceinline__ T grad() const {
    return grad_at<c, ka, false>(0, 0);
  }

  /* Second derivative along one kernel axis with Neumann ghost vertices. */
  template <int c, int ka> __device__ __forceinline__ T sd() const {
    const int di = ka == 0 ? 1 : 0, dj = ka == 0 ? 0 : 1;
    const T lo = v(c, -di, -dj), hi = v(c, di, dj), mid = v(c, 0, 0);
    T prev = lo, next = hi;
    if (ka == 0) {
      if (has_neu(0, c) && gi == 0) {
        const T g = face(m->neu, 0, c, gj);
        if (g == g) prev = hi - m->twod0 * g;
      }
      if (has_neu(1, c) && gi == m->nx - 1) {
        const T g = face(m->neu, 1, c, gj);
        if (g == g) next = lo + m->twod0 * g;
      }
      return ((next - T(2) * mid) + prev) * m->invdd0;
    } else {
      if (has_neu(2, c) && gj == 0) {
        const T g = face(m->neu, 2, c, gi);
        if (g == g) prev = hi - m->twod1 * g;
      }
      if (has_neu(3, c) && gj == m->ny - 1) {
        const T g = face(m->neu, 3, c, gi);
        if (g == g) next = lo + m->twod1 * g;
      }
      return ((next - T(2) * mid) + prev) * m->invdd1;
    }
  }

  /* Hessian element (kernel axes a1, a2). */
  template <int c, int a1, int a2> __device__ __forceinline__ T hess() const {
    if (a1 == a2) return sd<c, a1>();
    if (a2 == 0)
      return (grad_at<c, a1, true>(1, 0) - grad_at<c, a1, true>(-1, 0)) * m->inv2d0;
    return (grad_at<c, a1, true>(0, 1) - grad_at<c, a1, true>(0, -1)) * m->inv2d1;
  }
};

template <class Eq>
__device__ __forceinline__ constexpr bool has_dir(int f, int c) {
  return (Eq::DIR_MASK >> (f * Eq::C + c)) & 1ull;
}

/* Dirichlet re-imposition with the reference's face precedence. */
template <typename T, class Eq>
__device__ __forceinline__ T dirichlet(T v, int c, int gi, int gj, const MeshC<T>& m) {
  if (has_dir<Eq>(0, c) && gi == 0) {
    const T d = m.dir[(0 * Eq::C + c) * m.flen + gj];
    if (d == d) v = d;
  }
  if (has_dir<Eq>(1, c) && gi == m.nx - 1) {
    const T d = m.dir[(1 * Eq::C + c) * m.flen + gj];
    if (d == d) v = d;
  }
  if (has_dir<Eq>(2, c) && gj == 0) {
    const T d = m.dir[(2 * Eq::C + c) * m.flen + gi];
    if (d == d) v = d;
  }
  if (has_dir<Eq>(3, c) && gj == m.ny - 1) {
    const T d = m.dir[(3 * Eq::C + c) * m.flen + gi];
    if (d == d) v = d;
  }
  return v;
}

/* Whether any Dirichlet value constrains component c at (gi, gj). */
template <typename T, class Eq>
__device__ __forceinline__ bool dirichlet_applies(int c, int gi, int gj, const MeshC<T>& m) {
  bool hit = false;
  if (has_dir<Eq>(0, c) && gi == 0) hit |= m.dir[(0 * Eq::C + c) * m.flen + gj] == m.dir[(0 * Eq::C + c) * m.flen + gj];
  if (has_dir<Eq>(1, c) && gi == m.nx - 1) hit |= m.dir[(1 * Eq::C + c) * m.flen + gj] == m.dir[(1 * Eq::C + c) * m.flen + gj];
  if (has_dir<Eq>(2, c) && gj == 0) hit |= m.dir[(2 * Eq::C + c) * m.flen + gi] == m.dir[(2 * Eq::C + c) * m.flen + gi];
  if (has_dir<Eq>(3, c) && gj == m.ny - 1) hit |= m.dir[(3 * Eq::C + c) * m.flen + gi] == m.dir[(3 * Eq::C + c) * m.flen + gi];
  return hit;
}

/* r-th vertex of the ring of width h around a TX x TY tile, relative to the
 * tile origin. */
template <int TX, int TY>
__device__ __forceinline__ void ring_point(int h, int r, int& ti, int& tj) {
  const int w = TY + 2 * h;
  const int band = h * w;
  if (r < band) {
    ti = r / w - h;
    tj = r % w - h;
    return;
  }
  r -= band;
  if (r < band) {
    ti = TX + r / w;
    tj = r % w - h;
    return;
  }
  r -= band;
  const int hh = 2 * h;
  ti = r / hh;
  const int q = r - ti * hh;
  tj = q < h ? q - h : TY + (q - h);
}

template <int INTEG>
__device__ __forceinline__ constexpr double stage_time(int s) {
  return INTEG == RK4 ? (s == 0 ? 0.0 : (s == 3 ? 1.0 : 0.5))
                      : (INTEG == EXPLICIT_MIDPOINT ? (s == 0 ? 0.0 : 0.5) : 0.0);
}

template <typename T>
__device__ __forceinline__ T div6(T a) {
  /* (k1 + 2k2 + 2k3 + k4) / 6 as a product with the rounded reciprocal:
   * within one ulp of the quotient, and no IEEE division sequence */
  return a * T(1.0 / 6.0);
}

/* ---- TMA staging ---------------------------------------------------- */

/* A CUtensorMap (opaque, 128 bytes, 64-byte aligned), passed by value as a
 * __grid_constant__ kernel parameter. */
struct alignas(64) TmaDesc {
  unsigned long long w[16];
};

__device__ __forceinline__ unsigned smem_addr(const void* ptr) {
  return (unsigned)__cvta_generic_to_shared(ptr);
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

/* Waits for phase `parity` of the barrier for at most `limit_ns`. */
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > limit_ns) return false;
  }
  return true;
}

/* 5D tiled TMA load: box {cols, rows, C, 1, 1} at (x, y, 0, b, slot), zero
 * fill outside the tensor (the reference's zero halo). */
__device__ __forceinline__ void tma_load_5d(void* dst, const TmaDesc* map, int x, int y, int b,
                                            int slot, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(0), "r"(b), "r"(slot),
      "r"(smem_addr(bar))
      : "memory");
}

/* Column halo of the staged region: at least the stage count, rounded up
 * so that the first staged column starts on a 16-byte boundary (TMA). */
template <typename T, int NSTAGE>
struct ColHalo {
  static constexpr int align = 16 / (int)sizeof(T);
  static constexpr int value = ((NSTAGE + align - 1) / align) * align;
};

constexpr unsigned long long kWaitLimitNs = 2000000000ull; /* 2 s */

/* Stage-and-combine work of one tile whose input (tile + halo) is already
 * in `ybuf`.  MODE 0: one integrator step.  MODE 1: write the right-hand
 * side of every equation (dy/dt for D_Y_OVER_D_T rows, the value for LHS.Y
 * rows). */
template <typename T, class Eq, int INTEG, int TX, int TY, int NT, int MODE, int COMP = 0>
__device__ __forceinline__ void tile_compute(const prml_step_params& p, const MeshC<T>& m,
                                             const T* ybuf, T* bufA, T* bufB, int b, int gi0,
                                             int gj0) {
  constexpr int C = Eq::C;
  constexpr int ND = Eq::ND;
  constexpr int NSTAGE = (MODE == 1 || Eq::STAGE_INVARIANT) ? 1 : INTEG;
  constexpr int HX = NSTAGE;                    /* row halo */
  constexpr int HY = ColHalo<T, NSTAGE>::value; /* column halo */
  constexpr int RX = TX + 2 * HX, RY = TY + 2 * HY, RXY = RX * RY;
  constexpr int PER = (TX * TY) / NT;
  using P = Point<T, Eq, RY, RXY>;

  T* out = static_cast<T*>(p.out) + (long long)b * p.out_bstride;
  const double t0 = p.t + (p.t_offset ? p.t_offset[b] : 0.0);
  const T dt = T(p.dt);

  T acc[PER][ND > 0 ? ND : 1];
  const T* cur = ybuf;
  T* nxt = bufA;
  (void)bufB;

#pragma unroll
  for (int s = 0; s < NSTAGE; ++s) {
    const int h = NSTAGE - 1 - s;
    const double ts = t0 + stage_time<INTEG>(s) * p.dt;
    const bool last = (s == NSTAGE - 1);
    /* stage input of the next stage at region offset l (not used when last) */
    const double tn = t0 + stage_time<INTEG>(s + 1) * p.dt;
    (void)tn;

    auto stage_point = [&](int ti, int tj, int q) {
      const int li = HX + ti, lj = HY + tj;
      const int l = li * RY + lj;
      const int gi = gi0 + ti, gj = gj0 + tj;
      const bool inside = gi >= 0 && gi < p.nx && gj >= 0 && gj < p.ny;
      if (!inside) {
        if (!last) {
#pragma unroll
          for (int c = 0; c < C; ++c) nxt[c * RXY + l] = T(0);
        }
        return;
      }
      P pt{cur, l, gi, gj, &m, ts};
      if (MODE == 1) {
        T f[ND > 0 ? ND : 1];
        T g[Eq::NYC > 0 ? Eq::NYC : 1];
        if (ND > 0) Eq::rhs_dt(pt, f);
        if (Eq::NYC > 0) Eq::rhs_y(pt, g);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          T v = T(0);
#pragma unroll
          for (int i = 0; i < ND; ++i)
            if (Eq::dcomp(i) == c) v = f[i];
#pragma unroll
          for (int i = 0; i < Eq::NYC; ++i)
            if (Eq::ycomp(i) == c) v = g[i];
          out[c * p.cstride + (long long)gi * p.pitch + gj] = v;
        }
        return;
      }
      T f[ND > 0 ? ND : 1];
      if (ND > 0) Eq::rhs_dt(pt, f);
      if (!last) {
        /* next stage input: D components from the stage, others = c(y) */
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const T y = ybuf[c * RXY + l];
          T v = y;
#pragma unroll
          for (int i = 0; i < ND; ++i) {
            if (Eq::dcomp(i) == c) {
              if (INTEG == RK4) {
                const T k = dt * f[i];
                v = (s == 2) ? y + k : y + k * T(0.5);
              } else { /* explicit midpoint, s == 0 */
                v = y + (dt * T(0.5)) * f[i];
              }
            }
          }
          nxt[c * RXY + l] = dirichlet<T, Eq>(v, c, gi, gj, m);
        }
      }
      if (q >= 0) {
#pragma unroll
        for (int i = 0; i < ND; ++i) {
          if (INTEG == RK4) {
            const T k = dt * f[i];
            if (Eq::STAGE_INVARIANT) {
              acc[q][i] = ((k + T(2) * k) + T(2) * k) + k;
            } else if (s == 0) {
              acc[q][i] = k;
            } else if (s == 3) {
              acc[q][i] = acc[q][i] + k;
            } else {
              acc[q][i] = acc[q][i] + T(2) * k;
            }
          } else {
            acc[q][i] = dt * f[i];
          }
        }
      }
    };

#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int k = threadIdx.x + q * NT;
      const int ti = k / TY, tj = k - (k / TY) * TY;
      stage_point(ti, tj, q);
    }
    if (h > 0) {
      const int ring = 2 * h * (TY + 2 * h) + 2 * h * TX;
      for (int r = threadIdx.x; r < ring; r += NT) {
        int ti, tj;
        ring_point<TX, TY>(h, r, ti, tj);
        stage_point(ti, tj, -1);
      }
    }
    if (!last) {
      __syncthreads();
      cur = nxt;
      nxt = (nxt == bufA) ? bufB : bufA;
    }
  }
  if (MODE == 1) return;

  /* final combination, LHS.Y rows, Dirichlet, store */
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int k = threadIdx.x + q * NT;
    const int ti = k / TY, tj = k - (k / TY) * TY;
    const int gi = gi0 + ti, gj = gj0 + tj;
    if (gi >= p.nx || gj >= p.ny) continue;
    const int l = (HX + ti) * RY + (HY + tj);
    T yrhs[Eq::NYC > 0 ? Eq::NYC : 1];
    if (Eq::NYC > 0) {
      P pt{ybuf, l, gi, gj, &m, t0};
      Eq::rhs_y(pt, yrhs);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const T y = ybuf[c * RXY + l];
      const long long o = (long long)gi * p.pitch + gj;
      if (COMP) {
        /* compensated state: value = hi + lo, hi in planes [0, C), lo in
         * planes [C, 2C); the increment is added to (hi, lo) with an exact
         * two-sum so the rounding of every update is carried, not lost */
        T hi = y, lo = T(0);
        bool is_d = false;
#pragma unroll
        for (int i = 0; i < ND; ++i) {
          if (Eq::dcomp(i) == c) {
            is_d = true;
            const T* in_inst = static_cast<const T*>(p.in) + (long long)b * p.in_bstride;
            const T lo_in = in_inst[(C + c) * p.cstride + o];
            const T d = (INTEG == RK4) ? div6(acc[q][i]) : acc[q][i];
            const T t = d + lo_in;
            const T s = y + t;
            const T bb = s - y;
            lo = (y - (s - bb)) + (t - bb);
            hi = s;
          }
        }
#pragma unroll
        for (int i = 0; i < Eq::NYC; ++i)
          if (Eq::ycomp(i) == c) hi = yrhs[i];
        (void)is_d;
        const T dv = dirichlet<T, Eq>(hi, c, gi, gj, m);
        if (dirichlet_applies<T, Eq>(c, gi, gj, m)) lo = T(0);
        out[c * p.cstride + o] = dv;
        out[(C + c) * p.cstride + o] = lo;
        continue;
      }
      T v = y;
#pragma unroll
      for (int i = 0; i < ND; ++i)
        if (Eq::dcomp(i) == c) v = (INTEG == RK4) ? y + div6(acc[q][i]) : y + acc[q][i];
#pragma unroll
      for (int i = 0; i < Eq::NYC; ++i)
        if (Eq::ycomp(i) == c) v = yrhs[i];
      out[c * p.cstride + o] = dirichlet<T, Eq>(v, c, gi, gj, m);
    }
  }
}


/* Persistent step kernel body: the grid holds at most as many CTAs as fit
 * on the GPU at once, and each CTA walks the tiles (all instances, row-major
 * within an instance) with a stride of gridDim.x.  The input of the next
 * tile is fetched by TMA into the second staging buffer while the current
 * tile is computed, so load latency overlaps compute. */
template <typename T, class Eq, int INTEG, int TX, int TY, int NT, int MODE, int COMP = 0>
__device__ __forceinline__ void step_body(const prml_step_params& p, const TmaDesc& tin) {
  constexpr int C = Eq::C;
  constexpr int NSTAGE = (MODE == 1 || Eq::STAGE_INVARIANT) ? 1 : INTEG;
  constexpr int HX = NSTAGE;
  constexpr int HY = ColHalo<T, NSTAGE>::value;
  constexpr int RX = TX + 2 * HX, RY = TY + 2 * HY, RXY = RX * RY;
  constexpr int NSTG = NSTAGE == 1 ? 0 : (NSTAGE == 2 ? 1 : 2);
  static_assert((TX * TY) % NT == 0, "tile must be a multiple of the block");
  static_assert(C * 4 <= 64, "face masks hold at most 16 components");
  static_assert(RX <= 256 && RY <= 256, "TMA box extents are at most 256");
  constexpr unsigned kBoxBytes = (unsigned)(C * RXY * sizeof(T));

  /* every buffer starts on a 128-byte boundary: TMA destinations must */
  constexpr int BUF = (((C * RXY * (int)sizeof(T)) + 127) / 128) * 128 / (int)sizeof(T);
  extern __shared__ __align__(128) unsigned char prml_smem[];
  unsigned char* smem_base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(prml_smem) + 127ull) & ~127ull);
  T* ybuf0 = reinterpret_cast<T*>(smem_base);
  T* ybuf1 = ybuf0 + BUF;
  T* bufA = ybuf1 + BUF;
  T* bufB = bufA + BUF;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(ybuf0 + (2 + NSTG) * BUF);

  const int tiles_x = (p.ny + TY - 1) / TY;
  const int tiles_y = (p.nx + TX - 1) / TX;
  const int per_inst = tiles_x * tiles_y;
  const long long total = (long long)per_inst * p.batch;

  MeshC<T> m;
  m.inv2d0 = T(p.inv_2dx0);
  m.inv2d1 = T(p.inv_2dx1);
  m.invdd0 = T(p.inv_dxx0);
  m.invdd1 = T(p.inv_dxx1);
  m.twod0 = T(p.two_dx0);
  m.twod1 = T(p.two_dx1);
  m.nx = p.nx;
  m.ny = p.ny;
  m.flen = p.face_len;
  m.dir = static_cast<const T*>(p.dirichlet);
  m.neu = static_cast<const T*>(p.neumann);
  m.c0 = p.coord0;
  m.c1 = p.coord1;

  auto issue = [&](long long t, int buf) {
    const int b = (int)(t / per_inst);
    const int r = (int)(t - (long long)b * per_inst);
    const int ty = r / tiles_x, tx = r - ty * tiles_x;
    mbar_expect_tx(&bar[buf], kBoxBytes);
    tma_load_5d(buf ? ybuf1 : ybuf0, &tin, tx * TY - HY, ty * TX - HX, b, p.in_slot, &bar[buf]);
  };

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  __syncthreads();
  long long t = blockIdx.x;
  if (threadIdx.x == 0 && t < total) issue(t, 0);

  for (int it = 0; t < total; t += gridDim.x, ++it) {
    const int buf = it & 1;
    const long long next = t + gridDim.x;
    /* the other staging buffer was released by the __syncthreads that ended
     * the previous iteration */
    if (threadIdx.x == 0 && next < total) issue(next, buf ^ 1);
    const bool ok = mbar_wait_bounded(&bar[buf], (unsigned)((it >> 1) & 1), kWaitLimitNs);
    if (__syncthreads_or(!ok)) {
      /* a copy did not land in time: report, let in-flight copies finish
       * (bounded) so none outlives the CTA, then leave */
      if (threadIdx.x == 0 && p.status) atomicExch(p.status, 1);
      mbar_wait_bounded(&bar[buf], (unsigned)((it >> 1) & 1), kWaitLimitNs);
      if (next < total) mbar_wait_bounded(&bar[buf ^ 1], (unsigned)(((it + 1) >> 1) & 1), kWaitLimitNs);
      return;
    }
    const int b = (int)(t / per_inst);
    const int r = (int)(t - (long long)b * per_inst);
    const int ty = r / tiles_x, tx = r - ty * tiles_x;
    tile_compute<T, Eq, INTEG, TX, TY, NT, MODE, COMP>(p, m, buf ? ybuf1 : ybuf0, bufA, bufB, b,
                                                 ty * TX, tx * TY);
    __syncthreads();
  }
}

}  // namespace prml
