/*
 * Fused finite-difference step kernel (one launch = one full integrator step).
 *
 * Compiled at run time by NVRTC together with a generated equation struct
 * `Eq` (see pararealml_gb300/codegen.py).  One CTA owns a TX x TY tile of
 * output vertices of one instance.  It stages the tile plus a halo of HALO
 * vertices of every component of the input state in shared memory, then
 * evaluates the integrator's stages in shared memory on shrinking regions
 * (tile + HALO-1-s for stage s), so that every stage input is produced
 * on-chip and only the final state goes back to global memory.  Per step the
 * state is read once (plus halo) and written once.
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
__device__ __forceinline__ T div6(T a) { return a / T(6); }

/* MODE 0: one integrator step.  MODE 1: write the right-hand side of every
 * equation (dy/dt for D_Y_OVER_D_T rows, the value for LHS.Y rows). */
template <typename T, class Eq, int INTEG, int TX, int TY, int NT, int MODE>
__device__ __forceinline__ void step_body(const prml_step_params& p) {
  constexpr int C = Eq::C;
  constexpr int ND = Eq::ND;
  constexpr int NSTAGE = (MODE == 1 || Eq::STAGE_INVARIANT) ? 1 : INTEG;
  constexpr int HALO = NSTAGE;
  constexpr int RX = TX + 2 * HALO, RY = TY + 2 * HALO, RXY = RX * RY;
  constexpr int PER = (TX * TY) / NT;
  static_assert((TX * TY) % NT == 0, "tile must be a multiple of the block");
  static_assert(C * 4 <= 64, "face masks hold at most 16 components");
  using P = Point<T, Eq, RY, RXY>;

  extern __shared__ __align__(16) unsigned char prml_smem[];
  T* ybuf = reinterpret_cast<T*>(prml_smem);
  T* bufA = ybuf + C * RXY;
  T* bufB = bufA + C * RXY;

  const int b = blockIdx.z;
  const int gi0 = blockIdx.y * TX, gj0 = blockIdx.x * TY;

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

  const T* in = static_cast<const T*>(p.in) + (long long)b * p.in_bstride;
  T* out = static_cast<T*>(p.out) + (long long)b * p.out_bstride;
  const double t0 = p.t + (p.t_offset ? p.t_offset[b] : 0.0);
  const T dt = T(p.dt);

  /* 1. stage the tile + halo of every component, zero outside the domain */
  for (int e = threadIdx.x; e < C * RXY; e += NT) {
    const int c = e / RXY, r = e - c * RXY;
    const int li = r / RY, lj = r - li * RY;
    const int gi = gi0 - HALO + li, gj = gj0 - HALO + lj;
    T v = T(0);
    if (gi >= 0 && gi < p.nx && gj >= 0 && gj < p.ny)
      v = in[c * p.cstride + (long long)gi * p.pitch + gj];
    ybuf[e] = v;
  }
  __syncthreads();

  T acc[PER][ND > 0 ? ND : 1];
  const T* cur = ybuf;
  T* nxt = bufA;

#pragma unroll
  for (int s = 0; s < NSTAGE; ++s) {
    const int h = NSTAGE - 1 - s;
    const double ts = t0 + stage_time<INTEG>(s) * p.dt;
    const bool last = (s == NSTAGE - 1);
    /* stage input of the next stage at region offset l (not used when last) */
    const double tn = t0 + stage_time<INTEG>(s + 1) * p.dt;
    (void)tn;

    auto stage_point = [&](int ti, int tj, int q) {
      const int li = HALO + ti, lj = HALO + tj;
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
    const int l = (HALO + ti) * RY + (HALO + tj);
    T yrhs[Eq::NYC > 0 ? Eq::NYC : 1];
    if (Eq::NYC > 0) {
      P pt{ybuf, l, gi, gj, &m, t0};
      Eq::rhs_y(pt, yrhs);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const T y = ybuf[c * RXY + l];
      T v = y;
#pragma unroll
      for (int i = 0; i < ND; ++i)
        if (Eq::dcomp(i) == c) v = (INTEG == RK4) ? y + div6(acc[q][i]) : y + acc[q][i];
#pragma unroll
      for (int i = 0; i < Eq::NYC; ++i)
        if (Eq::ycomp(i) == c) v = yrhs[i];
      out[c * p.cstride + (long long)gi * p.pitch + gj] = dirichlet<T, Eq>(v, c, gi, gj, m);
    }
  }
}

}  // namespace prml
