/*
 * Fused FDM step kernels on 3D Cartesian meshes (compiled at run time by
 * NVRTC together with a generated `Eq` struct, like fdm_step.cuh).
 *
 * Kernel axes: 0 = planes (mesh axis 0, extent nz), 1 = rows (mesh axis 1,
 * nx), 2 = columns (mesh axis 2, ny, contiguous).  A state is
 * [instance][C][plane][row][pitch].  One CTA computes a TZ x TX x TY tile of
 * output vertices of one instance: ONE 5D TMA box load (columns, rows,
 * planes, components, instance x slot) stages the tile plus a halo of one
 * vertex per integrator stage (columns rounded up to 16 bytes), zero filled
 * outside the mesh, which is the reference's zero halo
 * (operators/fdm/numerical_differentiator.py:1012-1057).  The stages run in
 * shared memory on shrinking shells, exactly as the 2D kernels do.
 *
 * Faces: 2 ka + side for kernel axis ka.  A face is a 2D plane; its tables
 * are indexed by the two other kernel axes in C order: planes-face
 * (row, col), rows-face (plane, col), columns-face (plane, row), the order
 * of the reference's face constraint masks.
 */
#pragma once

#include "fdm_step.cuh"

namespace prml {

template <typename T>
struct MeshC3 {
  T inv2d[3], invdd[3], twod[3];
  T dd[3]; /* dx^2: divisors when Eq::EXACT_DIV */
  int n[3]; /* nz, nx, ny */
  int flen;
  const T* dir;
  const T* neu;
  const double* c[3];
  const float* cf[3];
};

/* index of vertex (k, i, j) within the face table of face f */
__device__ __forceinline__ int face_index3(int f, int k, int i, int j, const int (&n)[3]) {
  const int ka = f >> 1;
  return ka == 0 ? i * n[2] + j : (ka == 1 ? k * n[2] + j : k * n[1] + i);
}

template <typename T, class Eq, int RY, int RXY, int RV>
struct Point3 {
  using real = T;
  const T* s;
  int l;
  int g[3]; /* global (plane, row, col) */
  const MeshC3<T>* m;
  double time;

  __device__ __forceinline__ T v(int c, int d0, int d1, int d2) const {
    return s[c * RV + l + d0 * RXY + d1 * RY + d2];
  }
  static __device__ __forceinline__ constexpr bool has_neu(int f, int c) {
    return (Eq::NEU_MASK >> (f * Eq::C + c)) & 1ull;
  }
  __device__ __forceinline__ T face(const T* tab, int f, int c, int k, int i, int j) const {
    return tab[(f * Eq::C + c) * m->flen + face_index3(f, k, i, j, m->n)];
  }

  template <int c> __device__ __forceinline__ T val() const { return v(c, 0, 0, 0); }
  __device__ __forceinline__ T t() const { return T(time); }
  template <int ka> __device__ __forceinline__ T x() const {
    if constexpr (sizeof(T) == 4) return m->cf[ka][g[ka]];
    else return T(m->c[ka][g[ka]]);
  }

  /* first derivative along kernel axis ka at the vertex offset by d, with
   * the Neumann overwrite on the faces; zero outside the mesh when CHECK */
  template <int c, int ka, bool CHECK>
  __device__ __forceinline__ T grad_at(int d0, int d1, int d2) const {
    const int q0 = g[0] + d0, q1 = g[1] + d1, q2 = g[2] + d2;
    if (CHECK && (q0 < 0 || q0 >= m->n[0] || q1 < 0 || q1 >= m->n[1] || q2 < 0 || q2 >= m->n[2])) return T(0);
    const int q = ka == 0 ? q0 : (ka == 1 ? q1 : q2);
    if (has_neu(2 * ka, c) && q == 0) {
      const T gv = face(m->neu, 2 * ka, c, q0, q1, q2);
      if (gv == gv) return gv;
    }
    if (has_neu(2 * ka + 1, c) && q == m->n[ka] - 1) {
      const T gv = face(m->neu, 2 * ka + 1, c, q0, q1, q2);
      if (gv == gv) return gv;
    }
    const int e0 = ka == 0, e1 = ka == 1, e2 = ka == 2;
    if constexpr (Eq::EXACT_DIV) return (v(c, d0 + e0, d1 + e1, d2 + e2) - v(c, d0 - e0, d1 - e1, d2 - e2)) / m->twod[ka];
    return (v(c, d0 + e0, d1 + e1, d2 + e2) - v(c, d0 - e0, d1 - e1, d2 - e2)) * m->inv2d[ka];
  }
  template <int c, int ka> __device__ __forceinline__ T grad() const { return grad_at<c, ka, false>(0, 0, 0); }

  /* second derivative along kernel axis ka with Neumann ghost vertices */
  template <int c, int ka> __device__ __forceinline__ T sd() const {
    const int e0 = ka == 0, e1 = ka == 1, e2 = ka == 2;
    const T lo = v(c, -e0, -e1, -e2), hi = v(c, e0, e1, e2), mid = v(c, 0, 0, 0);
    T prev = lo, next = hi;
    if (has_neu(2 * ka, c) && g[ka] == 0) {
      const T gv = face(m->neu, 2 * ka, c, g[0], g[1], g[2]);
      if (gv == gv) prev = hi - m->twod[ka] * gv;
    }
    if (has_neu(2 * ka + 1, c) && g[ka] == m->n[ka] - 1) {
      const T gv = face(m->neu, 2 * ka + 1, c, g[0], g[1], g[2]);
      if (gv == gv) next = lo + m->twod[ka] * gv;
    }
    if constexpr (Eq::EXACT_DIV) return ((next - T(2) * mid) + prev) / m->dd[ka];
    return ((next - T(2) * mid) + prev) * m->invdd[ka];
  }

  /* Hessian element (kernel axes a1, a2): d/d a2 of the constrained d/d a1 */
  template <int c, int a1, int a2> __device__ __forceinline__ T hess() const {
    if (a1 == a2) return sd<c, a1>();
    const int e0 = a2 == 0, e1 = a2 == 1, e2 = a2 == 2;
    if constexpr (Eq::EXACT_DIV) return (grad_at<c, a1, true>(e0, e1, e2) - grad_at<c, a1, true>(-e0, -e1, -e2)) / m->twod[a2];
    return (grad_at<c, a1, true>(e0, e1, e2) - grad_at<c, a1, true>(-e0, -e1, -e2)) * m->inv2d[a2];
  }
};

/* Dirichlet re-imposition, later kernel axes win at edges and corners */
template <typename T, class Eq>
__device__ __forceinline__ T dirichlet3(T v, int c, const int (&g)[3], const MeshC3<T>& m) {
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    if (!((Eq::DIR_MASK >> (f * Eq::C + c)) & 1ull)) continue;
    const int ka = f >> 1;
    if (g[ka] != ((f & 1) ? m.n[ka] - 1 : 0)) continue;
    const T d = m.dir[(f * Eq::C + c) * m.flen + face_index3(f, g[0], g[1], g[2], m.n)];
    if (d == d) v = d;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ MeshC3<T> mesh3_at(const MeshC3<T>& m, const prml_step_params& p, int slot) {
  MeshC3<T> r = m;
  const long long off = (long long)slot * p.bc_stride;
  r.dir = m.dir + off;
  r.neu = m.neu + off;
  return r;
}

/* 5D TMA box (cols, rows, planes, components, instance x slot) */
__device__ __forceinline__ void tma_load_5d3(void* dst, const TmaDesc* map, int x, int y, int z, int bs,
                                             unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cta.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(0), "r"(bs),
      "r"(smem_addr(bar))
      : "memory");
}

/* Stages and combination of one staged tile (MODE 0: one step; MODE 1:
 * the right-hand sides).  Same schedule as the 2D tile_compute. */
template <typename T, class Eq, int INTEG, int TZ, int TX, int TY, int NT, int MODE>
__device__ __forceinline__ void tile_compute3(const prml_step_params& p, const MeshC3<T>& m, const T* ybuf,
                                              T* bufA, T* bufB, int b, int gk0, int gi0, int gj0) {
  constexpr int C = Eq::C;
  constexpr int ND = Eq::ND;
  constexpr int NSTAGE = (MODE == 1 || Eq::STAGE_INVARIANT) ? 1 : INTEG;
  constexpr int HZ = NSTAGE, HX = NSTAGE, HY = ColHalo<T, NSTAGE>::value;
  constexpr int RZ = TZ + 2 * HZ, RX = TX + 2 * HX, RY = TY + 2 * HY, RXY = RX * RY, RV = RZ * RXY;
  constexpr int PER = (TZ * TX * TY) / NT;
  using P = Point3<T, Eq, RY, RXY, RV>;

  T* out = static_cast<T*>(p.out) + (long long)b * p.out_bstride;
  const double t0 = Eq::USES_T ? p.t + (p.t_offset ? p.t_offset[b] : 0.0) : 0.0;
  const T dt = step_dt<T>(p);
  const long long plane = (long long)p.nx * p.pitch;

  T acc[PER][ND > 0 ? ND : 1];
  const T* cur = ybuf;
  T* nxt = bufA;
  (void)bufB;

#pragma unroll
  for (int s = 0; s < NSTAGE; ++s) {
    const int h = NSTAGE - 1 - s;
    const double ts = Eq::USES_T ? t0 + stage_time<INTEG>(s) * p.dt : 0.0;
    const bool last = (s == NSTAGE - 1);
    const MeshC3<T> ms = mesh3_at(m, p, bc_slot(p, b) + stage_half<INTEG>(s));
    const MeshC3<T> mn = mesh3_at(m, p, bc_slot(p, b) + (last ? 2 : stage_half<INTEG>(s + 1)));
    (void)mn;

    auto stage_point = [&](int tk, int ti, int tj, int q) {
      const int l = (HZ + tk) * RXY + (HX + ti) * RY + (HY + tj);
      const int g[3] = {gk0 + tk, gi0 + ti, gj0 + tj};
      const bool inside = g[0] >= 0 && g[0] < p.nz && g[1] >= 0 && g[1] < p.nx && g[2] >= 0 && g[2] < p.ny;
      if (!inside) {
        if (!last) {
#pragma unroll
          for (int c = 0; c < C; ++c) nxt[c * RV + l] = T(0);
        }
        return;
      }
      P pt{cur, l, {g[0], g[1], g[2]}, &ms, ts};
      if (MODE == 1) {
        T f[ND > 0 ? ND : 1];
        T gy[Eq::NYC > 0 ? Eq::NYC : 1];
        if (ND > 0) Eq::rhs_dt(pt, f);
        if (Eq::NYC > 0) Eq::rhs_y(pt, gy);
#pragma unroll
        for (int c = 0; c < C; ++c) {
          T v = T(0);
#pragma unroll
          for (int i = 0; i < ND; ++i)
            if (Eq::dcomp(i) == c) v = f[i];
#pragma unroll
          for (int i = 0; i < Eq::NYC; ++i)
            if (Eq::ycomp(i) == c) v = gy[i];
          out[c * p.cstride + g[0] * plane + (long long)g[1] * p.pitch + g[2]] = v;
        }
        return;
      }
      T f[ND > 0 ? ND : 1];
      if (ND > 0) Eq::rhs_dt(pt, f);
      if (!last) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const T y = ybuf[c * RV + l];
          T v = y;
#pragma unroll
          for (int i = 0; i < ND; ++i) {
            if (Eq::dcomp(i) == c) {
              if (INTEG == RK4) {
                const T k = dt * f[i];
                v = (s == 2) ? y + k : y + k * T(0.5);
              } else {
                v = y + (dt * T(0.5)) * f[i];
              }
            }
          }
          nxt[c * RV + l] = dirichlet3<T, Eq>(v, c, g, mn);
        }
      }
      if (q >= 0) {
#pragma unroll
        for (int i = 0; i < ND; ++i) {
          if (INTEG == RK4) {
            const T k = dt * f[i];
            if (Eq::STAGE_INVARIANT) acc[q][i] = ((k + T(2) * k) + T(2) * k) + k;
            else if (s == 0) acc[q][i] = k;
            else if (s == 3) acc[q][i] = acc[q][i] + k;
            else acc[q][i] = acc[q][i] + T(2) * k;
          } else {
            acc[q][i] = dt * f[i];
          }
        }
      }
    };

#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int k = threadIdx.x + q * NT;
      const int tk = k / (TX * TY), r = k - tk * (TX * TY);
      const int ti = r / TY, tj = r - ti * TY;
      stage_point(tk, ti, tj, q);
    }
    if (h > 0) {
      /* the shell of width h around the tile: walk the enlarged box and
       * skip the tile itself */
      constexpr int dummy = 0;
      (void)dummy;
      const int bz = TZ + 2 * h, bx = TX + 2 * h, by = TY + 2 * h;
      const int nbox = bz * bx * by;
      for (int r = threadIdx.x; r < nbox; r += NT) {
        const int tk = r / (bx * by) - h, rr = r % (bx * by);
        const int ti = rr / by - h, tj = rr % by - h;
        if (tk >= 0 && tk < TZ && ti >= 0 && ti < TX && tj >= 0 && tj < TY) continue;
        stage_point(tk, ti, tj, -1);
      }
    }
    if (!last) {
      __syncthreads();
      cur = nxt;
      nxt = (nxt == bufA) ? bufB : bufA;
    }
  }
  if (MODE == 1) return;

  /* final combination, LHS.Y rows (at t with the step-start Neumann values),
   * Dirichlet at t + dt, store */
  const MeshC3<T> m0 = mesh3_at(m, p, bc_slot(p, b));
  const MeshC3<T> m2 = mesh3_at(m, p, bc_slot(p, b) + 2);
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int k = threadIdx.x + q * NT;
    const int tk = k / (TX * TY), r = k - tk * (TX * TY);
    const int ti = r / TY, tj = r - ti * TY;
    const int g[3] = {gk0 + tk, gi0 + ti, gj0 + tj};
    if (g[0] >= p.nz || g[1] >= p.nx || g[2] >= p.ny) continue;
    const int l = (HZ + tk) * RXY + (HX + ti) * RY + (HY + tj);
    T yrhs[Eq::NYC > 0 ? Eq::NYC : 1];
    if (Eq::NYC > 0) {
      P pt{ybuf, l, {g[0], g[1], g[2]}, &m0, t0};
      Eq::rhs_y(pt, yrhs);
    }
    const long long o = g[0] * plane + (long long)g[1] * p.pitch + g[2];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const T y = ybuf[c * RV + l];
      T v = y;
#pragma unroll
      for (int i = 0; i < ND; ++i)
        if (Eq::dcomp(i) == c) v = (INTEG == RK4) ? y + div6(acc[q][i]) : y + acc[q][i];
#pragma unroll
      for (int i = 0; i < Eq::NYC; ++i)
        if (Eq::ycomp(i) == c) v = yrhs[i];
      out[c * p.cstride + o] = dirichlet3<T, Eq>(v, c, g, m2);
    }
  }
}

/* Persistent 3D step kernel body: CTAs walk the tiles (all instances) with
 * a stride of gridDim.x; the next tile's box is loaded by TMA into the
 * other staging buffer while the current one is computed. */
template <typename T, class Eq, int INTEG, int TZ, int TX, int TY, int NT, int MODE>
__device__ __forceinline__ void step_body3(const prml_step_params& p, const TmaDesc& tin) {
  constexpr int C = Eq::C;
  constexpr int NSTAGE = (MODE == 1 || Eq::STAGE_INVARIANT) ? 1 : INTEG;
  constexpr int HZ = NSTAGE, HX = NSTAGE, HY = ColHalo<T, NSTAGE>::value;
  constexpr int RZ = TZ + 2 * HZ, RX = TX + 2 * HX, RY = TY + 2 * HY;
  constexpr int NSTG = NSTAGE == 1 ? 0 : (NSTAGE == 2 ? 1 : 2);
  static_assert((TZ * TX * TY) % NT == 0, "tile must be a multiple of the block");
  static_assert(C * 6 <= 64, "face masks hold at most 10 components in 3D");
  static_assert(RX <= 256 && RY <= 256 && RZ <= 256, "TMA box extents are at most 256");
  constexpr unsigned kBoxBytes = (unsigned)(C * RZ * RX * RY * sizeof(T));
  constexpr int BUF = (((C * RZ * RX * RY * (int)sizeof(T)) + 127) / 128) * 128 / (int)sizeof(T);

  extern __shared__ __align__(128) unsigned char prml_smem[];
  unsigned char* smem_base = prml_smem + ((128u - (smem_addr(prml_smem) & 127u)) & 127u);
  T* ybuf0 = reinterpret_cast<T*>(smem_base);
  T* ybuf1 = ybuf0 + BUF;
  T* bufA = ybuf1 + BUF;
  T* bufB = bufA + BUF;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(ybuf0 + (2 + NSTG) * BUF);

  const int tiles_c = (p.ny + TY - 1) / TY;
  const int tiles_r = (p.nx + TX - 1) / TX;
  const int tiles_p = (p.nz + TZ - 1) / TZ;
  const int per_inst = tiles_c * tiles_r * tiles_p;
  const int total = per_inst * p.batch;

  MeshC3<T> m;
  const double i2[3] = {p.inv_2dx2, p.inv_2dx0, p.inv_2dx1};
  const double idd[3] = {p.inv_dxx2, p.inv_dxx0, p.inv_dxx1};
  const double tw[3] = {p.two_dx2, p.two_dx0, p.two_dx1};
  const float i2f[3] = {p.inv_2dx2_f, p.inv_2dx0_f, p.inv_2dx1_f};
  const float iddf[3] = {p.inv_dxx2_f, p.inv_dxx0_f, p.inv_dxx1_f};
  const float twf[3] = {p.two_dx2_f, p.two_dx0_f, p.two_dx1_f};
  const double ddd[3] = {p.dxx2, p.dxx0, p.dxx1};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if constexpr (sizeof(T) == 4) {
      m.inv2d[a] = i2f[a];
      m.invdd[a] = iddf[a];
      m.twod[a] = twf[a];
    } else {
      m.inv2d[a] = T(i2[a]);
      m.invdd[a] = T(idd[a]);
      m.twod[a] = T(tw[a]);
    }
    m.dd[a] = T(ddd[a]);
  }
  m.n[0] = p.nz;
  m.n[1] = p.nx;
  m.n[2] = p.ny;
  m.flen = p.face_len;
  m.dir = static_cast<const T*>(p.dirichlet);
  m.neu = static_cast<const T*>(p.neumann);
  m.c[0] = p.coord2;
  m.c[1] = p.coord0;
  m.c[2] = p.coord1;
  m.cf[0] = p.coord2_f;
  m.cf[1] = p.coord0_f;
  m.cf[2] = p.coord1_f;

  auto coords = [&](int t, int& b, int& tz, int& ty, int& tx) {
    b = t / per_inst;
    int r = t - b * per_inst;
    tz = r / (tiles_r * tiles_c);
    r -= tz * tiles_r * tiles_c;
    ty = r / tiles_c;
    tx = r - ty * tiles_c;
  };
  auto issue = [&](int t, int buf) {
    int b, tz, ty, tx;
    coords(t, b, tz, ty, tx);
    mbar_expect_tx(&bar[buf], kBoxBytes);
    tma_load_5d3(buf ? ybuf1 : ybuf0, &tin, tx * TY - HY, ty * TX - HX, tz * TZ - HZ,
                 p.in_slot * p.batch + b, &bar[buf]);
  };

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __syncthreads();
  int t = blockIdx.x;
  if (threadIdx.x == 0 && t < total) issue(t, 0);
  for (int it = 0; t < total; t += gridDim.x, ++it) {
    const int buf = it & 1;
    const int next = t + gridDim.x;
    if (threadIdx.x == 0 && next < total) issue(next, buf ^ 1);
    const unsigned long long wait_ns = p.wait_limit_ns ? p.wait_limit_ns : kWaitLimitNs;
    const bool ok = mbar_wait_bounded(&bar[buf], (unsigned)((it >> 1) & 1), wait_ns);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0 && p.status) atomicExch(p.status, 1);
      mbar_wait_bounded(&bar[buf], (unsigned)((it >> 1) & 1), wait_ns);
      if (next < total) mbar_wait_bounded(&bar[buf ^ 1], (unsigned)(((it + 1) >> 1) & 1), wait_ns);
      return;
    }
    int b, tz, ty, tx;
    coords(t, b, tz, ty, tx);
    tile_compute3<T, Eq, INTEG, TZ, TX, TY, NT, MODE>(p, m, buf ? ybuf1 : ybuf0, bufA, bufB, b, tz * TZ,
                                                     ty * TX, tx * TY);
    __syncthreads();
  }
}

}  // namespace prml
