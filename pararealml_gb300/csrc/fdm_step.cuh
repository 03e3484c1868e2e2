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
  T dd0, dd1; /* dx^2: divisors when Eq::EXACT_DIV */
  int nx, ny, flen;
  const T* dir;
  const T* neu;
  const double* c0;
  const double* c1;
  const float* c0f; /* float32 copies of c0, c1 */
  const float* c1f;
};

/* The boundary tables of half-step table `slot` (time t0 + slot dt / 2 of
 * the run).  Static conditions have bc_stride 0: every slot is the one
 * table. */
template <typename T>
__device__ __forceinline__ MeshC<T> mesh_at(const MeshC<T>& m, const prml_step_params& p, int slot) {
  MeshC<T> r = m;
  const long long off = (long long)slot * p.bc_stride;
  r.dir = m.dir + off;
  r.neu = m.neu + off;
  return r;
}

/* First boundary table of instance b in this launch: the launch's table
 * plus the instance's own offset (instances that start at different times
 * of one set of time-dependent tables, e.g. Parareal slices). */
__device__ __forceinline__ int bc_slot(const prml_step_params& p, int b) {
  return p.bc_slot0 + (p.bc_inst_slot ? p.bc_inst_slot[b] : 0);
}

/* Half steps from the step start to the time of integrator stage s
 * (RK4: t, t + dt/2, t + dt/2, t + dt; midpoint: t, t + dt/2). */
template <int INTEG>
__device__ __forceinline__ constexpr int stage_half(int s) {
  return INTEG == RK4 ? (s == 0 ? 0 : (s == 3 ? 2 : 1)) : (INTEG == EXPLICIT_MIDPOINT ? (s == 0 ? 0 : 1) : 0);
}

/* The step size in the state type: float32 kernels read the host-rounded
 * float copy and run no double arithmetic for it. */
template <typename T>
__device__ __forceinline__ T step_dt(const prml_step_params& p) {
  if constexpr (sizeof(T) == 4) return p.dt_f;
  else return T(p.dt);
}

/* a * b + c with one rounding.  Modules are compiled without automatic
 * contraction (so that kernel variants round alike); fused-order modules
 * (Eq::FAST) place their multiply-adds explicitly with this. */
template <typename T>
__device__ __forceinline__ T fmaT(T a, T b, T c) {
  if constexpr (sizeof(T) == 4) return __fmaf_rn(a, b, c);
  else return __fma_rn(a, b, c);
}

/* A vertex of the current stage input, with the stencil operators the
 * generated right-hand sides call. */
template <typename T, class Eq, int RY, int RXY, bool EDGE = true>
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
    if constexpr (sizeof(T) == 4) return ka == 0 ? m->c0f[gi] : m->c1f[gj];
    else return ka == 0 ? T(m->c0[gi]) : T(m->c1[gj]);
  }

  /* Constrained first derivative along kernel axis ka at the vertex offset
   * by (di, dj); zero outside the domain when CHECK is set. */
  template <int c, int ka, bool CHECK>
  __device__ __forceinline__ T grad_at(int di, int dj) const {
    const int qi = gi + di, qj = gj + dj;
    if (EDGE && CHECK && (qi < 0 || qi >= m->nx || qj < 0 || qj >= m->ny)) return T(0);
    if (ka == 0) {
      if (EDGE && has_neu(0, c) && qi == 0) {
        const T g = face(m->neu, 0, c, qj);
        if (g == g) return g;
      }
      if (EDGE && has_neu(1, c) && qi == m->nx - 1) {
        const T g = face(m->neu, 1, c, qj);
        if (g == g) return g;
      }
      if constexpr (Eq::EXACT_DIV) return (v(c, di + 1, dj) - v(c, di - 1, dj)) / m->twod0;
      return (v(c, di + 1, dj) - v(c, di - 1, dj)) * m->inv2d0;
    } else {
      if (EDGE && has_neu(2, c) && qj == 0) {
        const T g = face(m->neu, 2, c, qi);
        if (g == g) return g;
      }
      if (EDGE && has_neu(3, c) && qj == m->ny - 1) {
        const T g = face(m->neu, 3, c, qi);
        if (g == g) return g;
      }
      if constexpr (Eq::EXACT_DIV) return (v(c, di, dj + 1) - v(c, di, dj - 1)) / m->twod1;
      return (v(c, di, dj + 1) - v(c, di, dj - 1)) * m->inv2d1;
    }
  }
  template <int c, int ka> __device__ __forceinline__ T grad() const {
    return grad_at<c, ka, false>(0, 0);
  }

  /* Neighbours (prev, next) of the vertex along one kernel axis, with the
   * Neumann ghost vertices y[1] - 2dx g (lower face) and y[n-2] + 2dx g
   * (upper face) of _add_halos_along_axis where a value is given. */
  template <int c, int ka> __device__ __forceinline__ void ends(T& prev, T& next) const {
    const int di = ka == 0 ? 1 : 0, dj = ka == 0 ? 0 : 1;
    const T lo = v(c, -di, -dj), hi = v(c, di, dj);
    prev = lo;
    next = hi;
    if (ka == 0) {
      if (EDGE && has_neu(0, c) && gi == 0) {
        const T g = face(m->neu, 0, c, gj);
        if (g == g) prev = hi - m->twod0 * g;
      }
      if (EDGE && has_neu(1, c) && gi == m->nx - 1) {
        const T g = face(m->neu, 1, c, gj);
        if (g == g) next = lo + m->twod0 * g;
      }
    } else {
      if (EDGE && has_neu(2, c) && gj == 0) {
        const T g = face(m->neu, 2, c, gi);
        if (g == g) prev = hi - m->twod1 * g;
      }
      if (EDGE && has_neu(3, c) && gj == m->ny - 1) {
        const T g = face(m->neu, 3, c, gi);
        if (g == g) next = lo + m->twod1 * g;
      }
    }
  }

  /* Second derivative along one kernel axis with Neumann ghost vertices. */
  template <int c, int ka> __device__ __forceinline__ T sd() const {
    const T mid = v(c, 0, 0);
    T prev, next;
    ends<c, ka>(prev, next);
    if (ka == 0) {
      if constexpr (Eq::EXACT_DIV) return ((next - T(2) * mid) + prev) / m->dd0;
      return ((next - T(2) * mid) + prev) * m->invdd0;
    } else {
      if constexpr (Eq::EXACT_DIV) return ((next - T(2) * mid) + prev) / m->dd1;
      return ((next - T(2) * mid) + prev) * m->invdd1;
    }
  }

  /* Laplacian over both kernel axes (the sum of the two second derivatives
   * of sd) in fused order: the four neighbours summed first, the centre
   * subtracted with one multiply-add, one scaling when both axes share a
   * step size.  Used by fused-order modules (Eq::FAST) only. */
  template <int c> __device__ __forceinline__ T lap() const {
    const T mid = v(c, 0, 0);
    T p0, n0, p1, n1;
    ends<c, 0>(p0, n0);
    ends<c, 1>(p1, n1);
    if constexpr (Eq::EQUAL_DX) return fmaT(T(-4), mid, (n0 + p0) + (n1 + p1)) * m->invdd0;
    else return fmaT(fmaT(T(-2), mid, n0 + p0), m->invdd0, fmaT(T(-2), mid, n1 + p1) * m->invdd1);
  }

  /* The same Laplacian unscaled (both axes share the step size): the
   * generated code multiplies it by inv_dd() as part of its term's constant
   * coefficient, which the compiler computes once per thread, so a scaled
   * Laplacian term costs one multiplication per vertex instead of two. */
  template <int c> __device__ __forceinline__ T lapr() const {
    const T mid = v(c, 0, 0);
    T p0, n0, p1, n1;
    ends<c, 0>(p0, n0);
    ends<c, 1>(p1, n1);
    return fmaT(T(-4), mid, (n0 + p0) + (n1 + p1));
  }
  __device__ __forceinline__ T inv_dd() const { return m->invdd0; }

  /* Hessian element (kernel axes a1, a2). */
  template <int c, int a1, int a2> __device__ __forceinline__ T hess() const {
    if (a1 == a2) return sd<c, a1>();
    if constexpr (Eq::EXACT_DIV) {
      if (a2 == 0) return (grad_at<c, a1, true>(1, 0) - grad_at<c, a1, true>(-1, 0)) / m->twod0;
      return (grad_at<c, a1, true>(0, 1) - grad_at<c, a1, true>(0, -1)) / m->twod1;
    }
    if (a2 == 0)
      return (grad_at<c, a1, true>(1, 0) - grad_at<c, a1, true>(-1, 0)) * m->inv2d0;
    return (grad_at<c, a1, true>(0, 1) - grad_at<c, a1, true>(0, -1)) * m->inv2d1;
  }
};

template <class Eq>
__device__ __forceinline__ constexpr bool has_dir(int f, int c) {
  return (Eq::DIR_MASK >> (f * Eq::C + c)) & 1ull;
}

/* Dirichlet re-imposition with the reference's face precedence.  EDGE =
 * false: the vertex is known to be off every face (interior tile). */
template <typename T, class Eq, bool EDGE = true>
__device__ __forceinline__ T dirichlet(T v, int c, int gi, int gj, const MeshC<T>& m) {
  if (!EDGE) return v;
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
template <typename T, class Eq, bool EDGE = true>
__device__ __forceinline__ bool dirichlet_applies(int c, int gi, int gj, const MeshC<T>& m) {
  if (!EDGE) return false;
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

/* One try_wait that suspends the thread in hardware (up to suspend_ns, a
 * hint) until the phase completes, so waiting warps do not spin. */
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity,
                                              unsigned suspend_ns) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(suspend_ns)
      : "memory");
  return ok != 0;
}
/* Waits for the phase with the given parity for at most limit_ns: the first
 * try costs no clock read; the clock bounds the rare long waits. */
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns) {
  constexpr unsigned kSuspendNs = 1000000u; /* 1 ms per try */
  if (mbar_try_wait(bar, parity, kSuspendNs)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity, kSuspendNs)) {
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

/* Per-vertex integrator arithmetic of the multi-stage kernels
 * (numerical_integrator.py:65-132), in one place so every stage walk over
 * it rounds alike.  Next stage input of a D component: y + (dt / 2) f, or
 * y + dt f for RK4's third stage. */
template <typename T, class Eq, int INTEG>
__device__ __forceinline__ T stage_input(T y, T f, T dt, int s) {
  if constexpr (Eq::FAST) {
    return fmaT((INTEG == RK4 && s == 2) ? dt : dt * T(0.5), f, y);
  } else if constexpr (INTEG == RK4) {
    const T k = dt * f;
    return (s == 2) ? y + k : y + k * T(0.5);
  } else { /* explicit midpoint, s == 0 */
    return y + (dt * T(0.5)) * f;
  }
}

/* Stage slope accumulation.  Fused order: slopes accumulated unscaled (f1 +
 * 2 f2 + 2 f3 + f4 for RK4, the last stage's slope otherwise) and scaled
 * once in step_result; reference order: the reference's k sums. */
template <typename T, class Eq, int INTEG>
__device__ __forceinline__ void stage_accumulate(T& acc, T f, T dt, int s) {
  if constexpr (Eq::FAST) {
    if (INTEG == RK4 && s > 0) acc = (s == 3) ? acc + f : fmaT(T(2), f, acc);
    else acc = f;
  } else if constexpr (INTEG == RK4) {
    const T k = dt * f;
    if (Eq::STAGE_INVARIANT) acc = ((k + T(2) * k) + T(2) * k) + k;
    else if (s == 0) acc = k;
    else if (s == 3) acc = acc + k;
    else acc = acc + T(2) * k;
  } else {
    acc = dt * f;
  }
}

/* The step's result from the accumulated slopes (acc_scale: dt / 6 for
 * RK4, dt otherwise; fused order only). */
template <typename T, class Eq, int INTEG>
__device__ __forceinline__ T step_result(T y, T acc, T acc_scale) {
  if constexpr (Eq::FAST) return fmaT(acc_scale, acc, y);
  else return (INTEG == RK4) ? y + div6(acc) : y + acc;
}

/* Stage-and-combine work of one tile whose input (tile + halo) is already
 * in `ybuf`.  MODE 0: one integrator step.  MODE 1: write the right-hand
 * side of every equation (dy/dt for D_Y_OVER_D_T rows, the value for LHS.Y
 * rows). */
template <typename T, class Eq, int INTEG, int TX, int TY, int NT, int MODE, int COMP, bool EDGE>
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
  using P = Point<T, Eq, RY, RXY, EDGE>;

  T* out = static_cast<T*>(p.out) + (long long)b * p.out_bstride;
  /* time in double only for right-hand sides that read t */
  const double t0 = Eq::USES_T ? p.t + (p.t_offset ? p.t_offset[b] : 0.0) : 0.0;
  const T dt = step_dt<T>(p);
  const int slot0 = bc_slot(p, b);

  T acc[PER][ND > 0 ? ND : 1];
  const T* cur = ybuf;
  T* nxt = bufA;
  (void)bufB;

#pragma unroll
  for (int s = 0; s < NSTAGE; ++s) {
    const int h = NSTAGE - 1 - s;
    const double ts = Eq::USES_T ? t0 + stage_time<INTEG>(s) * p.dt : 0.0;
    const bool last = (s == NSTAGE - 1);

    /* the reference evaluates the Neumann values at the stage time and
     * constrains each stage input (and the result) at its own time */
    const MeshC<T> ms = mesh_at(m, p, slot0 + stage_half<INTEG>(s));
    const MeshC<T> mn = mesh_at(m, p, slot0 + (last ? 2 : stage_half<INTEG>(s + 1)));
    (void)mn;
    auto stage_point = [&](int ti, int tj, int q) {
      const int li = HX + ti, lj = HY + tj;
      const int l = li * RY + lj;
      const int gi = gi0 + ti, gj = gj0 + tj;
      const bool inside = !EDGE || (gi >= 0 && gi < p.nx && gj >= 0 && gj < p.ny);
      if (!inside) {
        if (!last) {
#pragma unroll
          for (int c = 0; c < C; ++c) nxt[c * RXY + l] = T(0);
        }
        return;
      }
      P pt{cur, l, gi, gj, &ms, ts};
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
          for (int i = 0; i < ND; ++i)
            if (Eq::dcomp(i) == c) v = stage_input<T, Eq, INTEG>(y, f[i], dt, s);
          nxt[c * RXY + l] = dirichlet<T, Eq, EDGE>(v, c, gi, gj, mn);
        }
      }
      if (q >= 0) {
#pragma unroll
        for (int i = 0; i < ND; ++i) stage_accumulate<T, Eq, INTEG>(acc[q][i], f[i], dt, s);
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

  /* final combination, LHS.Y rows, Dirichlet, store: LHS.Y right-hand
   * sides at (t, y) with the step-start Neumann values, every result
   * constrained at t + dt */
  const MeshC<T> m0 = mesh_at(m, p, slot0);
  const MeshC<T> m2 = mesh_at(m, p, slot0 + 2);
  /* fused order: the accumulated slopes' scale (RK4: dt / 6) */
  const T acc_scale = INTEG == RK4 ? dt * T(1.0 / 6.0) : dt;
  (void)acc_scale;
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int k = threadIdx.x + q * NT;
    const int ti = k / TY, tj = k - (k / TY) * TY;
    const int gi = gi0 + ti, gj = gj0 + tj;
    if (EDGE && (gi >= p.nx || gj >= p.ny)) continue;
    const int l = (HX + ti) * RY + (HY + tj);
    T yrhs[Eq::NYC > 0 ? Eq::NYC : 1];
    if (Eq::NYC > 0) {
      P pt{ybuf, l, gi, gj, &m0, t0};
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
            const T d = Eq::FAST ? acc_scale * acc[q][i] : ((INTEG == RK4) ? div6(acc[q][i]) : acc[q][i]);
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
        const T dv = dirichlet<T, Eq, EDGE>(hi, c, gi, gj, m2);
        if (dirichlet_applies<T, Eq, EDGE>(c, gi, gj, m2)) lo = T(0);
        out[c * p.cstride + o] = dv;
        out[(C + c) * p.cstride + o] = lo;
        continue;
      }
      T v = y;
#pragma unroll
      for (int i = 0; i < ND; ++i)
        if (Eq::dcomp(i) == c) v = step_result<T, Eq, INTEG>(y, acc[q][i], acc_scale);
#pragma unroll
      for (int i = 0; i < Eq::NYC; ++i)
        if (Eq::ycomp(i) == c) v = yrhs[i];
      out[c * p.cstride + o] = dirichlet<T, Eq, EDGE>(v, c, gi, gj, m2);
    }
  }
}

/* Single-stage time steps on one staged tile, in one pass per step: the
 * right-hand sides, the LHS.Y values, the combination, the Dirichlet values
 * and the store of each vertex together.  TB > 1 (temporal blocking):
 * `p.tb_steps` (<= TB) single-stage time steps
 * (forward Euler, or any integrator whose stages are identical: see
 * STAGE_INVARIANT) on one staged tile whose halo is TB vertices deep.  Step s
 * of the block computes the tile plus a ring of TB-1-s vertices, so each
 * step's values at the ring are exactly the values the neighbouring tiles
 * compute for their own vertices, and the tile's values equal TB single
 * steps.  Every step's tile interior is stored (to tb_out[j], or `out` for
 * the last step); the ring values only feed the next step in shared memory.
 * COMP = 1: compensated float32 state (hi planes [0, C), lo planes [C, 2C);
 * the lo planes are staged with the halo when TB > 1, else read at the
 * vertex), updated with an exact two-sum per step. */
template <typename T, class Eq, int INTEG, int TX, int TY, int NT, int TB, int COMP, bool EDGE>
__device__ __forceinline__ void tile_compute_tb(const prml_step_params& p, const MeshC<T>& m,
                                                const T* ybuf, T* bufA, T* bufB, int b, int gi0,
                                                int gj0) {
  constexpr int C = Eq::C;
  constexpr int ND = Eq::ND;
  constexpr int PL = COMP ? 2 * C : C; /* staged planes */
  constexpr int HX = TB;
  constexpr int HY = ColHalo<T, TB>::value;
  constexpr int RX = TX + 2 * HX, RY = TY + 2 * HY, RXY = RX * RY;
  constexpr int PER = (TX * TY) / NT;
  using P = Point<T, Eq, RY, RXY, EDGE>;
  static_assert(Eq::STAGE_INVARIANT || INTEG == FORWARD_EULER, "temporal blocking needs single-stage steps");

  /* one step per launch is known at compile time: no step loop remains */
  const int nsteps = TB == 1 ? 1 : (p.tb_steps < 1 ? 1 : (p.tb_steps > TB ? TB : p.tb_steps));
  const int s0 = TB - nsteps;
  const double tb0 = Eq::USES_T ? p.t + (p.t_offset ? p.t_offset[b] : 0.0) : 0.0;
  const T dt = step_dt<T>(p);
  const int slot0 = bc_slot(p, b);
  const T* cur = ybuf;
  T* nxt = bufA;

  for (int s = s0; s < TB; ++s) {
    const int h = TB - 1 - s;
    const int j = s - s0;
    const bool last = (s == TB - 1);
    const double ts = Eq::USES_T ? tb0 + (double)j * p.dt : 0.0;
    T* dst = last ? static_cast<T*>(p.out) + (long long)b * p.out_bstride
                  : (p.tb_out[j] ? static_cast<T*>(p.tb_out[j]) + (long long)b * p.tb_bstride : nullptr);
    /* Neumann values at the step start, Dirichlet values at its end */
    const MeshC<T> ms = mesh_at(m, p, slot0 + 2 * j);
    const MeshC<T> me = mesh_at(m, p, slot0 + 2 * j + 2);

    auto step_point = [&](int ti, int tj, bool interior) {
      const int l = (HX + ti) * RY + (HY + tj);
      const int gi = gi0 + ti, gj = gj0 + tj;
      const bool inside = !EDGE || (gi >= 0 && gi < p.nx && gj >= 0 && gj < p.ny);
      if (!inside) {
        if (!last) {
#pragma unroll
          for (int c = 0; c < PL; ++c) nxt[c * RXY + l] = T(0);
        }
        return;
      }
      P pt{cur, l, gi, gj, &ms, ts};
      /* fused order: f[i] = fk[i] * (the rest of dy/dt), fk[i] the product
       * of the term's constant factors (1 if none), so that the update is
       * one multiply-add by dt fk[i], computed once per thread */
      T f[ND > 0 ? ND : 1];
      T fk[ND > 0 ? ND : 1];
      if constexpr (ND > 0) {
        if constexpr (Eq::FAST && !COMP) {
          Eq::rhs_dt_split(pt, f, fk);
        } else {
          Eq::rhs_dt(pt, f);
#pragma unroll
          for (int i = 0; i < ND; ++i) fk[i] = T(1);
        }
      }
      T yrhs[Eq::NYC > 0 ? Eq::NYC : 1];
      if (Eq::NYC > 0) Eq::rhs_y(pt, yrhs);
      const long long o = (long long)gi * p.pitch + gj;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const T y = cur[c * RXY + l];
        T hi = y, lo = T(0);
#pragma unroll
        for (int i = 0; i < ND; ++i) {
          if (Eq::dcomp(i) == c) {
            const T k = dt * (fk[i] * f[i]);
            /* fused order: a stage-invariant RK4 step is y + dt f (the
             * reference's ((k + 2k) + 2k + k) / 6 equals k up to rounding) */
            const T d = (INTEG == RK4 && !Eq::FAST) ? div6(((k + T(2) * k) + T(2) * k) + k) : k;
            if constexpr (COMP) {
              /* lo of the step input: staged with the halo when blocked,
               * else read at the vertex itself */
              T lo_in;
              if constexpr (TB == 1)
                lo_in = static_cast<const T*>(p.in)[(long long)b * p.in_bstride + (C + c) * p.cstride + o];
              else
                lo_in = cur[(C + c) * RXY + l];
              const T t = d + lo_in;
              const T sm = y + t;
              const T bb = sm - y;
              lo = (y - (sm - bb)) + (t - bb);
              hi = sm;
            } else {
              hi = Eq::FAST ? fmaT(dt * fk[i], f[i], y) : y + d;
            }
          }
        }
#pragma unroll
        for (int i = 0; i < Eq::NYC; ++i)
          if (Eq::ycomp(i) == c) hi = yrhs[i];
        const T v = dirichlet<T, Eq, EDGE>(hi, c, gi, gj, me);
        if (COMP && dirichlet_applies<T, Eq, EDGE>(c, gi, gj, me)) lo = T(0);
        if (!last) {
          nxt[c * RXY + l] = v;
          if (COMP) nxt[(C + c) * RXY + l] = lo;
        }
        if (interior && (last || dst)) {
          dst[c * p.cstride + o] = v;
          if (COMP) dst[(C + c) * p.cstride + o] = lo;
        }
      }
    };

#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int k = threadIdx.x + q * NT;
      const int ti = k / TY, tj = k - (k / TY) * TY;
      if (!EDGE || (gi0 + ti < p.nx && gj0 + tj < p.ny)) step_point(ti, tj, true);
      else if (!last) step_point(ti, tj, false);
    }
    if (h > 0) {
      const int ring = 2 * h * (TY + 2 * h) + 2 * h * TX;
      for (int r = threadIdx.x; r < ring; r += NT) {
        int ti, tj;
        ring_point<TX, TY>(h, r, ti, tj);
        step_point(ti, tj, false);
      }
    }
    if (!last) {
      __syncthreads();
      cur = nxt;
      nxt = (nxt == bufA) ? bufB : bufA;
    }
  }
}

/* Persistent step kernel body: the grid holds at most as many CTAs as fit
 * on the GPU at once, and each CTA walks the tiles (all instances, row-major
 * within an instance) with a stride of gridDim.x.  The input of the next
 * tile is fetched by TMA into the second staging buffer while the current
 * tile is computed, so load latency overlaps compute. */
template <typename T, class Eq, int INTEG, int TX, int TY, int NT, int MODE, int COMP = 0, int TB = 1>
__device__ __forceinline__ void step_body(const prml_step_params& p, const TmaDesc& tin) {
  constexpr int C = Eq::C;
  constexpr int NSTAGE = (MODE == 1 || Eq::STAGE_INVARIANT) ? 1 : INTEG;
  static_assert(TB == 1 || (MODE == 0 && NSTAGE == 1), "temporal blocking needs single-stage steps");
  static_assert(TB >= 1 && TB <= PRML_TB_MAX, "temporal block out of range");
  constexpr int HX = TB > 1 ? TB : NSTAGE;
  constexpr int HY = ColHalo<T, HX>::value;
  constexpr int RX = TX + 2 * HX, RY = TY + 2 * HY, RXY = RX * RY;
  /* on-chip buffers besides the two staging buffers: stage (or step) inputs */
  constexpr int NSTG = TB > 1 ? (TB == 2 ? 1 : 2) : (NSTAGE == 1 ? 0 : (NSTAGE == 2 ? 1 : 2));
  /* staged planes: a blocked compensated state carries its lo planes too */
  constexpr int PL = (TB > 1 && COMP) ? 2 * C : C;
  static_assert((TX * TY) % NT == 0, "tile must be a multiple of the block");
  static_assert(C * 4 <= 64, "face masks hold at most 16 components");
  static_assert(RX <= 256 && RY <= 256, "TMA box extents are at most 256");
  constexpr unsigned kBoxBytes = (unsigned)(PL * RXY * sizeof(T));

  /* every buffer starts on a 128-byte boundary: TMA destinations must */
  constexpr int BUF = (((PL * RXY * (int)sizeof(T)) + 127) / 128) * 128 / (int)sizeof(T);
  extern __shared__ __align__(128) unsigned char prml_smem[];
  /* round up to 128 bytes by offsetting the shared array itself (not via an
   * integer round trip), so the compiler keeps every staged access in the
   * shared address space */
  unsigned char* smem_base = prml_smem + ((128u - (smem_addr(prml_smem) & 127u)) & 127u);
  T* ybuf0 = reinterpret_cast<T*>(smem_base);
  T* ybuf1 = ybuf0 + BUF;
  T* bufA = ybuf1 + BUF;
  T* bufB = bufA + BUF;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(ybuf0 + (2 + NSTG) * BUF);

  const int tiles_x = (p.ny + TY - 1) / TY;
  const int tiles_y = (p.nx + TX - 1) / TX;
  const int per_inst = tiles_x * tiles_y;
  const int total = per_inst * p.batch; /* the host keeps this below 2^31 */

  /* Tile walk with a stride of gridDim.x tiles and no division per tile:
   * the stride is split once into (instances, rows, columns) of tiles and
   * added with carries (each part is below its extent, so one carry each). */
  struct Walk {
    int b, ty, tx;
  };
  const int G = (int)gridDim.x;
  const int gb = G / per_inst, gr = G - gb * per_inst;
  const int gy = gr / tiles_x, gx = gr - gy * tiles_x;
  auto advance = [&](Walk w) {
    w.tx += gx;
    int c = w.tx >= tiles_x;
    w.tx -= c ? tiles_x : 0;
    w.ty += gy + c;
    c = w.ty >= tiles_y;
    w.ty -= c ? tiles_y : 0;
    w.b += gb + c;
    return w;
  };

  MeshC<T> m;
  if constexpr (sizeof(T) == 4) {
    m.inv2d0 = p.inv_2dx0_f;
    m.inv2d1 = p.inv_2dx1_f;
    m.invdd0 = p.inv_dxx0_f;
    m.invdd1 = p.inv_dxx1_f;
    m.twod0 = p.two_dx0_f;
    m.twod1 = p.two_dx1_f;
  } else {
    m.inv2d0 = T(p.inv_2dx0);
    m.inv2d1 = T(p.inv_2dx1);
    m.invdd0 = T(p.inv_dxx0);
    m.invdd1 = T(p.inv_dxx1);
    m.twod0 = T(p.two_dx0);
    m.twod1 = T(p.two_dx1);
  }
  m.dd0 = T(p.dxx0);
  m.dd1 = T(p.dxx1);
  m.c0f = p.coord0_f;
  m.c1f = p.coord1_f;
  m.nx = p.nx;
  m.ny = p.ny;
  m.flen = p.face_len;
  m.dir = static_cast<const T*>(p.dirichlet);
  m.neu = static_cast<const T*>(p.neumann);
  m.c0 = p.coord0;
  m.c1 = p.coord1;

  const unsigned long long wait_ns = p.wait_limit_ns ? p.wait_limit_ns : kWaitLimitNs;
  auto issue = [&](const Walk& w, int buf) {
    mbar_expect_tx(&bar[buf], kBoxBytes);
    if (!p.wait_probe)
      tma_load_5d(buf ? ybuf1 : ybuf0, &tin, w.tx * TY - HY, w.ty * TX - HX, w.b, p.in_slot, &bar[buf]);
  };

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  /* programmatic dependent launch: the next step may start its CTAs now;
   * this one waits for its predecessor to complete (and its writes to be
   * visible) before any global memory access.  Both are no-ops when the
   * launch did not ask for the overlap. */
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __syncthreads();
  int t = blockIdx.x;
  Walk cur;
  cur.b = t / per_inst;
  cur.ty = (t - cur.b * per_inst) / tiles_x;
  cur.tx = t - cur.b * per_inst - cur.ty * tiles_x;
  Walk nxt = advance(cur);
  if (threadIdx.x == 0 && t < total) issue(cur, 0);

  for (int it = 0; t < total; t += G, ++it) {
    const int buf = it & 1;
    const int next = t + G;
    /* the other staging buffer was released by the __syncthreads that ended
     * the previous iteration */
    if (threadIdx.x == 0 && next < total) issue(nxt, buf ^ 1);
    const bool ok = mbar_wait_bounded(&bar[buf], (unsigned)((it >> 1) & 1), wait_ns);
    if (__syncthreads_or(!ok)) {
      /* a copy did not land in time: report, let in-flight copies finish
       * (bounded) so none outlives the CTA, then leave */
      if (threadIdx.x == 0 && p.status) atomicExch(p.status, 1);
      mbar_wait_bounded(&bar[buf], (unsigned)((it >> 1) & 1), wait_ns);
      if (next < total) mbar_wait_bounded(&bar[buf ^ 1], (unsigned)(((it + 1) >> 1) & 1), wait_ns);
      return;
    }
    const int b = cur.b;
    const int gi0 = cur.ty * TX, gj0 = cur.tx * TY;
    /* interior tile: every vertex it evaluates (tile + ring), and every
     * neighbour a mixed derivative reaches, is off the mesh faces, so the
     * face (Neumann, Dirichlet) and inside tests compile away */
    const bool edge = gi0 < HX + 1 || gi0 + TX + HX + 1 > p.nx || gj0 < HX + 1 || gj0 + TY + HX + 1 > p.ny;
    const T* ybuf = buf ? ybuf1 : ybuf0;
    if constexpr (MODE == 0 && NSTAGE == 1) {
      /* single-stage steps (one or TB per launch): one pass per step */
      if (edge) tile_compute_tb<T, Eq, INTEG, TX, TY, NT, TB, COMP, true>(p, m, ybuf, bufA, bufB, b, gi0, gj0);
      else tile_compute_tb<T, Eq, INTEG, TX, TY, NT, TB, COMP, false>(p, m, ybuf, bufA, bufB, b, gi0, gj0);
    } else {
      if (edge) tile_compute<T, Eq, INTEG, TX, TY, NT, MODE, COMP, true>(p, m, ybuf, bufA, bufB, b, gi0, gj0);
      else tile_compute<T, Eq, INTEG, TX, TY, NT, MODE, COMP, false>(p, m, ybuf, bufA, bufB, b, gi0, gj0);
    }
    __syncthreads();
    cur = nxt;
    nxt = advance(nxt);
  }
}

/* Mesh constants of a launch in the state type (float32 kernels read the
 * host-rounded float copies). */
template <typename T>
__device__ __forceinline__ MeshC<T> make_mesh(const prml_step_params& p) {
  MeshC<T> m;
  if constexpr (sizeof(T) == 4) {
    m.inv2d0 = p.inv_2dx0_f;
    m.inv2d1 = p.inv_2dx1_f;
    m.invdd0 = p.inv_dxx0_f;
    m.invdd1 = p.inv_dxx1_f;
    m.twod0 = p.two_dx0_f;
    m.twod1 = p.two_dx1_f;
  } else {
    m.inv2d0 = T(p.inv_2dx0);
    m.inv2d1 = T(p.inv_2dx1);
    m.invdd0 = T(p.inv_dxx0);
    m.invdd1 = T(p.inv_dxx1);
    m.twod0 = T(p.two_dx0);
    m.twod1 = T(p.two_dx1);
  }
  m.dd0 = T(p.dxx0);
  m.dd1 = T(p.dxx1);
  m.c0f = p.coord0_f;
  m.c1f = p.coord1_f;
  m.nx = p.nx;
  m.ny = p.ny;
  m.flen = p.face_len;
  m.dir = static_cast<const T*>(p.dirichlet);
  m.neu = static_cast<const T*>(p.neumann);
  m.c0 = p.coord0;
  m.c1 = p.coord1;
  return m;
}

/* 16 bytes of state (4 floats or 2 doubles) read through L2 only: the
 * state was written by the previous launch, which may still have been
 * running when this one started (programmatic dependent launch), so no
 * L1 copy is trusted. */
__device__ __forceinline__ void ld16(const float* a, float* d) {
  const float4 v = __ldcg(reinterpret_cast<const float4*>(a));
  d[0] = v.x;
  d[1] = v.y;
  d[2] = v.z;
  d[3] = v.w;
}
__device__ __forceinline__ void ld16(const double* a, double* d) {
  const double2 v = __ldcg(reinterpret_cast<const double2*>(a));
  d[0] = v.x;
  d[1] = v.y;
}
__device__ __forceinline__ void st16(float* a, const float* d) {
  *reinterpret_cast<float4*>(a) = make_float4(d[0], d[1], d[2], d[3]);
}
__device__ __forceinline__ void st16(double* a, const double* d) {
  *reinterpret_cast<double2*>(a) = make_double2(d[0], d[1]);
}

/* One tile of the register-window step (see walk_body): the thread's
 * window rows gi0 - 1 .. gi0 + R, columns gj0 - 1 .. gj0 + VW of every
 * component (zero outside the mesh), then its R x VW vertices. */
template <typename T, class Eq, int INTEG, int R, int COMP, bool EDGE>
__device__ __forceinline__ void walk_tile(const prml_step_params& p, const MeshC<T>& m, int b, int gi0,
                                          int gj0, int g) {
  constexpr int C = Eq::C;
  constexpr int ND = Eq::ND;
  constexpr int VW = 16 / (int)sizeof(T);
  constexpr int NR = R + 2, NC = VW + 2, NRC = NR * NC;
  using P = Point<T, Eq, NC, NRC, EDGE>;

  const T* in = static_cast<const T*>(p.in) + (long long)b * p.in_bstride;
  T* out = static_cast<T*>(p.out) + (long long)b * p.out_bstride;
  const bool cols_in = gj0 < p.ny; /* the thread's vector starts inside the mesh */

  T w[C * NRC];
#pragma unroll
  for (int c = 0; c < C; ++c) {
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const int gi = gi0 - 1 + r;
      T* row = w + c * NRC + r * NC;
      const T* src = in + c * p.cstride + (long long)gi * p.pitch + gj0;
      const bool row_in = !EDGE || (gi >= 0 && gi < p.nx);
      if (row_in && (!EDGE || cols_in)) {
        ld16(src, row + 1);
      } else {
#pragma unroll
        for (int k = 0; k < VW; ++k) row[1 + k] = T(0);
      }
      if (EDGE) {
        /* the reference's zero halo: columns past the mesh read 0 (the
         * row padding holds no state) */
#pragma unroll
        for (int k = 0; k < VW; ++k)
          if (gj0 + k >= p.ny) row[1 + k] = T(0);
      }
      /* the neighbouring columns come from the neighbouring lanes of the
       * group of 8; the group's first and last lanes read theirs */
      T left = __shfl_up_sync(0xffffffffu, row[VW], 1, 8);
      T right = __shfl_down_sync(0xffffffffu, row[1], 1, 8);
      if (g == 0) left = (row_in && (!EDGE || (gj0 >= 1 && gj0 - 1 < p.ny))) ? __ldcg(src - 1) : T(0);
      if (g == 7) right = (row_in && (!EDGE || gj0 + VW < p.ny)) ? __ldcg(src + VW) : T(0);
      row[0] = left;
      row[NC - 1] = right;
    }
  }

  const double tb0 = Eq::USES_T ? p.t + (p.t_offset ? p.t_offset[b] : 0.0) : 0.0;
  const T dt = step_dt<T>(p);
  const int slot0 = bc_slot(p, b);
  /* Neumann values at the step start, Dirichlet values at its end */
  const MeshC<T> ms = mesh_at(m, p, slot0);
  const MeshC<T> me = mesh_at(m, p, slot0 + 2);

#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int gi = gi0 + r;
    if (EDGE && gi >= p.nx) break;
    T res[C][VW];
    T lo[C][VW];
    T lo_in[C][VW];
    if constexpr (COMP) {
#pragma unroll
      for (int c = 0; c < C; ++c) {
        if (cols_in) ld16(in + (C + c) * p.cstride + (long long)gi * p.pitch + gj0, lo_in[c]);
        else
#pragma unroll
          for (int k = 0; k < VW; ++k) lo_in[c][k] = T(0);
      }
    }
#pragma unroll
    for (int k = 0; k < VW; ++k) {
      const int gj = gj0 + k;
#pragma unroll
      for (int c = 0; c < C; ++c) res[c][k] = lo[c][k] = T(0);
      if (EDGE && gj >= p.ny) continue;
      const int l = (1 + r) * NC + 1 + k;
      P pt{w, l, gi, gj, &ms, tb0};
      T f[ND > 0 ? ND : 1];
      T fk[ND > 0 ? ND : 1];
      if constexpr (ND > 0) {
        if constexpr (Eq::FAST && !COMP) {
          Eq::rhs_dt_split(pt, f, fk);
        } else {
          Eq::rhs_dt(pt, f);
#pragma unroll
          for (int i = 0; i < ND; ++i) fk[i] = T(1);
        }
      }
      T yrhs[Eq::NYC > 0 ? Eq::NYC : 1];
      if (Eq::NYC > 0) Eq::rhs_y(pt, yrhs);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const T y = w[c * NRC + l];
        T hi = y, lo_c = T(0);
#pragma unroll
        for (int i = 0; i < ND; ++i) {
          if (Eq::dcomp(i) == c) {
            if constexpr (COMP) {
              const T kk = dt * (fk[i] * f[i]);
              const T d = (INTEG == RK4 && !Eq::FAST) ? div6(((kk + T(2) * kk) + T(2) * kk) + kk) : kk;
              const T t = d + lo_in[c][k];
              const T sm = y + t;
              const T bb = sm - y;
              lo_c = (y - (sm - bb)) + (t - bb);
              hi = sm;
            } else if constexpr (Eq::FAST) {
              hi = fmaT(dt * fk[i], f[i], y);
            } else {
              const T kk = dt * f[i];
              hi = y + ((INTEG == RK4) ? div6(((kk + T(2) * kk) + T(2) * kk) + kk) : kk);
            }
          }
        }
#pragma unroll
        for (int i = 0; i < Eq::NYC; ++i)
          if (Eq::ycomp(i) == c) hi = yrhs[i];
        res[c][k] = dirichlet<T, Eq, EDGE>(hi, c, gi, gj, me);
        if (COMP && dirichlet_applies<T, Eq, EDGE>(c, gi, gj, me)) lo_c = T(0);
        lo[c][k] = lo_c;
      }
    }
    if (EDGE && !cols_in) continue;
    const long long o = (long long)gi * p.pitch + gj0;
    if (!EDGE || gj0 + VW <= p.ny) {
#pragma unroll
      for (int c = 0; c < C; ++c) {
        st16(out + c * p.cstride + o, res[c]);
        if (COMP) st16(out + (C + c) * p.cstride + o, lo[c]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < VW; ++k) {
        if (gj0 + k >= p.ny) break;
#pragma unroll
        for (int c = 0; c < C; ++c) {
          out[c * p.cstride + o + k] = res[c][k];
          if (COMP) out[(C + c) * p.cstride + o + k] = lo[c][k];
        }
      }
    }
  }
}

/* Register-window step kernel for single-stage steps (forward Euler, or a
 * system whose integrator stages coincide): no staging, no shared memory,
 * no barrier.  A tile is TX = 4 R rows by TY = NW 8 VW columns (VW = 16
 * bytes of state); warp w of the CTA takes the tile's columns
 * [8 VW w, 8 VW (w + 1)), and its lane (q, g) = (lane / 8, lane % 8) the
 * VW columns from 8 VW w + VW g and the R rows from q R.  Every thread reads
 * its R + 2 rows of VW + 2 columns of each component from global memory
 * (one 16-byte load per row, the two neighbouring columns from the
 * neighbouring lanes) into registers and evaluates the generated
 * right-hand sides with the same Point as the staged kernels over that
 * window (RY = VW + 2), so both round alike.  The CTAs walk the tiles with
 * a stride of the grid, as step_body does. */
template <typename T, class Eq, int INTEG, int R, int NW, int COMP>
__device__ __forceinline__ void walk_body(const prml_step_params& p) {
  constexpr int VW = 16 / (int)sizeof(T);
  constexpr int TX = 4 * R, TY = NW * 8 * VW;
  static_assert(Eq::STAGE_INVARIANT || INTEG == FORWARD_EULER, "register-window steps need single-stage steps");
  const int tiles_x = (p.ny + TY - 1) / TY;
  const int tiles_y = (p.nx + TX - 1) / TX;
  const int per_inst = tiles_x * tiles_y;
  const int total = per_inst * p.batch;
  const MeshC<T> m = make_mesh<T>(p);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int q = lane >> 3, g = lane & 7;

  /* tile walk with a stride of the grid, advanced with carries (no
   * division per tile), as in step_body */
  const int G = (int)gridDim.x;
  const int gb = G / per_inst, gr = G - gb * per_inst;
  const int gy = gr / tiles_x, gx = gr - gy * tiles_x;
  int t = blockIdx.x;
  int b = t / per_inst;
  int ty = (t - b * per_inst) / tiles_x;
  int tx = t - b * per_inst - ty * tiles_x;

  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  for (; t < total; t += G) {
    const int ri = ty * TX, cw = tx * TY + wid * 8 * VW;
    /* warps whose columns lie past the mesh have nothing to do */
    if (cw < p.ny) {
      /* interior warp: its vertices and their neighbours are off the faces */
      const bool edge = ri < 2 || ri + TX + 2 > p.nx || cw < 2 || cw + 8 * VW + 2 > p.ny;
      const int gi0 = ri + q * R, gj0 = cw + g * VW;
      if (edge) walk_tile<T, Eq, INTEG, R, COMP, true>(p, m, b, gi0, gj0, g);
      else walk_tile<T, Eq, INTEG, R, COMP, false>(p, m, b, gi0, gj0, g);
    }
    tx += gx;
    int c = tx >= tiles_x;
    tx -= c ? tiles_x : 0;
    ty += gy + c;
    c = ty >= tiles_y;
    ty -= c ? tiles_y : 0;
    b += gb + c;
  }
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* a) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
  return v;
}

/* Grid-wide barrier of a cooperative launch: a monotonic arrival counter
 * (zero at launch), `target` = CTAs x barriers passed so far.  Every thread's
 * global stores are ordered before the tensor (async proxy) loads other CTAs
 * issue after the barrier.  The wait is bounded by %globaltimer; false when
 * it gave up. */
__device__ __forceinline__ bool grid_barrier(unsigned long long* cnt, unsigned long long target,
                                             unsigned long long limit_ns) {
  asm volatile("fence.proxy.async.global;" ::: "memory");
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(cnt, 1ull);
    bool ok = true;
    if (ld_acquire_u64(cnt) < target) {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_u64(cnt) < target) {
        __nanosleep(64);
        if (global_ns() - t0 > limit_ns) {
          ok = false;
          break;
        }
      }
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return s_ok != 0;
}

/* Multi-round persistent kernel body (one cooperative launch, see
 * prml_multi_params): every round takes one step of each group that has
 * steps left.  The round's tiles (all groups, all instances, row-major
 * within an instance) are walked with a stride of gridDim.x as in
 * step_body, the next tile staged by TMA while the current one computes;
 * a grid barrier separates the rounds, so a step reads the halo its
 * neighbours wrote in the previous round.  Every group uses this kernel's
 * tile, stage schedule and state type. */
template <typename T, class Eq, int INTEG, int TX, int TY, int NT, int COMP = 0>
__device__ __forceinline__ void multi_body(const prml_multi_params& mp) {
  constexpr int C = Eq::C;
  constexpr int NSTAGE = Eq::STAGE_INVARIANT ? 1 : INTEG;
  constexpr int HX = NSTAGE;
  constexpr int HY = ColHalo<T, HX>::value;
  constexpr int RX = TX + 2 * HX, RY = TY + 2 * HY, RXY = RX * RY;
  constexpr int NSTG = NSTAGE == 1 ? 0 : (NSTAGE == 2 ? 1 : 2);
  static_assert((TX * TY) % NT == 0, "tile must be a multiple of the block");
  static_assert(RX <= 256 && RY <= 256, "TMA box extents are at most 256");
  constexpr unsigned kBoxBytes = (unsigned)(C * RXY * sizeof(T));
  constexpr int BUF = (((C * RXY * (int)sizeof(T)) + 127) / 128) * 128 / (int)sizeof(T);
  extern __shared__ __align__(128) unsigned char prml_smem[];
  unsigned char* smem_base = prml_smem + ((128u - (smem_addr(prml_smem) & 127u)) & 127u);
  T* ybuf0 = reinterpret_cast<T*>(smem_base);
  T* ybuf1 = ybuf0 + BUF;
  T* bufA = ybuf1 + BUF;
  T* bufB = bufA + BUF;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(ybuf0 + (2 + NSTG) * BUF);

  __shared__ prml_step_params sp[PRML_MULTI_MAX_GROUPS];
  __shared__ int s_first[PRML_MULTI_MAX_GROUPS + 1]; /* first item of each group this round */
  __shared__ int s_map[PRML_MULTI_MAX_GROUPS];       /* tensor map of each group's input */
  const int ng = mp.n_groups;
  const TmaDesc* maps = static_cast<const TmaDesc*>(mp.maps);
  if ((int)threadIdx.x < ng) sp[threadIdx.x] = mp.groups[threadIdx.x].p;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  __syncthreads();

  const int G = (int)gridDim.x;
  unsigned q = 0; /* tiles staged so far by this CTA: buffer q & 1, phase (q >> 1) & 1 */
  /* the first group's wait bound (0 = 2 s); its wait_probe 2 (error-path
   * tests only) makes every grid barrier wait for one arrival more than
   * the grid has, so the first barrier runs out after that bound */
  const unsigned long long wait_ns = sp[0].wait_limit_ns ? sp[0].wait_limit_ns : kWaitLimitNs;
  const unsigned long long extra = sp[0].wait_probe == 2 ? 1ull : 0ull;

  struct Item {
    int g, b, ty, tx;
  };
  auto locate = [&](int t) {
    Item it;
    int g = 0;
    while (g + 1 < ng && s_first[g + 1] <= t) ++g;
    const prml_multi_group& grp = mp.groups[g];
    const int per_inst = grp.tiles_x * grp.tiles_y;
    const int local = t - s_first[g];
    it.g = g;
    it.b = local / per_inst;
    const int rem = local - it.b * per_inst;
    it.ty = rem / grp.tiles_x;
    it.tx = rem - it.ty * grp.tiles_x;
    return it;
  };
  auto issue = [&](const Item& w, int buf) {
    mbar_expect_tx(&bar[buf], kBoxBytes);
    tma_load_5d(buf ? ybuf1 : ybuf0, &maps[s_map[w.g]], w.tx * TY - HY, w.ty * TX - HX, w.b, sp[w.g].in_slot,
                &bar[buf]);
  };

  for (int r = 0; r < mp.n_rounds; ++r) {
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int g = 0; g < ng; ++g) {
        const prml_multi_group& grp = mp.groups[g];
        s_first[g] = acc;
        if (r < grp.n_steps) {
          prml_step_params& p = sp[g];
          const long long es = p.elem_bytes;
          if (r == 0) {
            p.in = grp.first;
            p.in_slot = 0;
            s_map[g] = 2 * g;
          } else {
            const int in_slot = grp.ping_pong ? ((r - 1) & 1) : (r - 1);
            p.in = static_cast<const char*>(grp.main) + (long long)in_slot * grp.slot_stride * es;
            p.in_slot = in_slot;
            s_map[g] = 2 * g + 1;
          }
          const int out_slot = grp.ping_pong ? (r & 1) : r;
          p.out = static_cast<char*>(grp.main) + (long long)out_slot * grp.slot_stride * es;
          p.t = grp.t0 + (double)r * p.dt;
          p.bc_slot0 = 2 * r;
          p.tb_steps = 1;
          acc += p.batch * grp.tiles_x * grp.tiles_y;
        }
      }
      s_first[ng] = acc;
    }
    __syncthreads();
    const int total = s_first[ng];
    int t = blockIdx.x;
    Item cur = t < total ? locate(t) : Item{0, 0, 0, 0};
    if (threadIdx.x == 0 && t < total) issue(cur, q & 1);
    for (; t < total; t += G, ++q) {
      const int buf = q & 1;
      const int next = t + G;
      Item nxt = next < total ? locate(next) : cur;
      if (threadIdx.x == 0 && next < total) issue(nxt, buf ^ 1);
      const bool ok = mbar_wait_bounded(&bar[buf], (q >> 1) & 1, wait_ns);
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0 && mp.status) atomicExch(mp.status, 1);
        mbar_wait_bounded(&bar[buf], (q >> 1) & 1, wait_ns);
        if (next < total) mbar_wait_bounded(&bar[buf ^ 1], ((q + 1) >> 1) & 1, wait_ns);
        return;
      }
      /* by value: only the fields the tile reads become registers, and the
       * staging stores (generic pointers into shared memory) cannot force
       * them to be reloaded as a reference into the shared table would */
      const prml_step_params p = sp[cur.g];
      const MeshC<T> m = make_mesh<T>(p);
      const int gi0 = cur.ty * TX, gj0 = cur.tx * TY;
      const bool edge = gi0 < HX + 1 || gi0 + TX + HX + 1 > p.nx || gj0 < HX + 1 || gj0 + TY + HX + 1 > p.ny;
      const T* ybuf = buf ? ybuf1 : ybuf0;
      if constexpr (NSTAGE == 1) {
        if (edge) tile_compute_tb<T, Eq, INTEG, TX, TY, NT, 1, COMP, true>(p, m, ybuf, bufA, bufB, cur.b, gi0, gj0);
        else tile_compute_tb<T, Eq, INTEG, TX, TY, NT, 1, COMP, false>(p, m, ybuf, bufA, bufB, cur.b, gi0, gj0);
      } else {
        if (edge) tile_compute<T, Eq, INTEG, TX, TY, NT, 0, COMP, true>(p, m, ybuf, bufA, bufB, cur.b, gi0, gj0);
        else tile_compute<T, Eq, INTEG, TX, TY, NT, 0, COMP, false>(p, m, ybuf, bufA, bufB, cur.b, gi0, gj0);
      }
      __syncthreads();
      cur = nxt;
    }
    if (r + 1 < mp.n_rounds &&
        !grid_barrier(mp.barrier, (unsigned long long)(r + 1) * (unsigned long long)G + extra, wait_ns)) {
      if (threadIdx.x == 0 && mp.status) atomicExch(mp.status, 1);
      return;
    }
  }
}

}  // namespace prml
