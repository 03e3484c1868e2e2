/*
 * pararealml_gb300 — C ABI of the GB300 (sm_103a) FDM + Parareal engine.
 *
 * The reference (ViktorC/PararealML) is pure Python and has no FFI; the entry
 * points below are what its hot path would bind through ctypes to replace the
 * numpy kernels named beside each group.  All pointers are device pointers
 * unless stated, all sizes are element counts, streams are cudaStream_t
 * passed as void*, and every function returns 0 on success or one of the
 * PRML_ERR_* codes, with the message available from prml_last_error().
 * No C++ exception and no torch type crosses this boundary.
 */
#ifndef PARAREALML_GB300_H
#define PARAREALML_GB300_H

#include "prml_params.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PRML_ABI_VERSION 1

#define PRML_OK 0
#define PRML_ERR_ARG 1       /* invalid argument (reference: ValueError)      */
#define PRML_ERR_COMPILE 2   /* run-time compilation of a generated module    */
#define PRML_ERR_CUDA 3      /* CUDA driver/runtime failure                   */
#define PRML_ERR_UNSUPPORTED 4
#define PRML_ERR_CONVERGENCE 5 /* an iterative solve hit its iteration cap  */

/* Message of the last failure on the calling thread (never NULL). */
const char* prml_last_error(void);
int prml_abi_version(void);
/* sizeof(prml_step_params), so bindings can check their mirror of it. */
int prml_step_params_size(void);

/* ---- run-time compiled stencil modules --------------------------------
 * Replaces the per-equation right-hand-side construction of the reference:
 * SymbolMapper.create_rhs_map_function / sympy.lambdify
 * (pararealml/operators/symbol_mapper.py:222-253) and
 * FDMSymbolMapper (pararealml/operators/fdm/fdm_symbol_mapper.py:26-158).
 * `source` is CUDA C++ generated from the equation system; it is compiled
 * for `arch` (e.g. "sm_103a") with the ';'-separated include directories and
 * the space-separated extra NVRTC options, and the cubin is written to
 * `cache_path` (an existing cubin there is reused). */
int prml_jit_compile(const char* source, const char* include_dirs, const char* arch,
                     const char* extra_options, const char* cache_path, char* log,
                     long long log_len);
int prml_module_load(const char* cubin_path, void** module_out);
int prml_module_unload(void* module);
/* Looks up an extern "C" kernel and sets its dynamic shared memory size. */
int prml_module_kernel(void* module, const char* name, int smem_bytes, void** kernel_out);
int prml_kernel_free(void* kernel);
int prml_kernel_occupancy(void* kernel, int block, int* blocks_per_sm);

/* ---- FDM time stepping ------------------------------------------------
 * Replaces the step loop of FDMOperator.solve
 * (pararealml/operators/fdm/fdm_operator.py:48-77) together with
 * NumericalIntegrator.integral (numerical_integrator.py:42-132) and the
 * ThreePointCentralDifferenceMethod stencils (numerical_differentiator.py:
 * 999-1242).  Runs n_steps fused step kernels starting from y0; step s
 * (1-based) is written to traj + (s/save_every - 1) * traj_step_stride when
 * save_every divides s, else to one of the two work buffers.  `base` holds
 * the mesh, boundary tables and strides; in/out/t/dt are filled per step.
 * Inputs are staged by TMA: every state buffer gets a 5D tensor map with a
 * (box_rows x box_cols x comps) box, the staged tile + halo of the kernel;
 * buffers must be 16-byte aligned with 16-byte-multiple strides. */
int prml_fdm_run(void* kernel, int block, int tile_x, int tile_y, int box_rows, int box_cols,
                 int comps, const prml_step_params* base, const void* y0, long long y0_bstride,
                 void* traj, long long traj_bstride, long long traj_step_stride,
                 void* work_a, void* work_b, long long work_bstride, long long n_steps,
                 int save_every, double t0, double dt, void* stream);
/* Evaluates the right-hand side of every equation at (t, y) into f
 * (reference: FDMSymbolMapper.map_concatenated, fdm_symbol_mapper.py:150-158). */
int prml_fdm_rhs(void* kernel, int block, int tile_x, int tile_y, int box_rows, int box_cols,
                 int comps, const prml_step_params* base, const void* y, long long y_bstride,
                 void* f, long long f_bstride, double t, void* stream);
/* Step launches overlap (programmatic dependent launch): each step kernel
 * lets the next start its CTAs early and waits for its predecessor before
 * any global memory access.  No reference counterpart (the reference's step
 * loop is Python, fdm_operator.py:66-72).  Returns the previous setting;
 * on by default. */
int prml_set_step_overlap(int enabled);

/* ---- multi-round launches ---------------------------------------------
 * Replace the step loop of FDMOperator.solve (fdm_operator.py:66-72) for
 * several independent solves at once, as the reference runs them one
 * FDMOperator.solve call after another: ONE persistent cooperative launch of
 * a generated `prml_multi_*` kernel takes every step of every group (see
 * prml_multi_group in prml_params.h), round r being step r of each group
 * with more than r steps, a grid-wide barrier between rounds (bounded:
 * after 2 s of waiting the kernel sets *status and returns).
 * prml_multi_prepare encodes the groups' tensor maps and copies the
 * descriptors into the caller's device buffer `desc` (at least
 * prml_multi_desc_bytes(n_groups) bytes, 128-byte aligned; synchronous, so
 * call it before any stream capture).  prml_multi_launch zeroes the barrier
 * counter (a device unsigned long long) on `stream` and launches with at
 * most one CTA per resident slot and no more CTAs than max_round_tiles (the
 * largest round's tile count); both steps can be recorded in a CUDA graph. */
/* sizeof(prml_multi_group), so bindings can check their mirror of it. */
int prml_multi_group_size(void);
long long prml_multi_desc_bytes(int n_groups);
int prml_multi_prepare(const prml_multi_group* groups, int n_groups, int tile_x, int tile_y, int box_rows,
                       int box_cols, int comps, void* desc, long long desc_bytes);
int prml_multi_launch(void* kernel, int block, const void* desc, int n_groups, int n_rounds,
                      long long max_round_tiles, unsigned long long* barrier, int* status, int max_ctas,
                      void* stream);

/* ---- anti-Laplacian (Jacobi) -------------------------------------------
 * Replaces NumericalDifferentiator.anti_laplacian and
 * ThreePointCentralDifferenceMethod._next_anti_laplacian_estimate
 * (pararealml/operators/fdm/numerical_differentiator.py:872-927,
 * 1097-1186), which FDMOperator calls once per step for the LHS.Y_LAPLACIAN
 * components (fdm_operator.py:141-161).  Per instance: starting from y_init
 * (constrained), repeat y <- constrained Jacobi estimate while the 2-norm
 * of the change over all solved components exceeds tol, starting from an
 * infinite change (tol = inf runs no iteration).  Kernel axes: 0 = planes, 1 = rows, 2 = columns;
 * a mesh of dimension d uses axes [3 - d, 3). */
typedef struct prml_jacobi_params {
  int n[3];            /* vertices per kernel axis (1 where the mesh has none)  */
  int first_axis;      /* 3 - mesh dimension                                    */
  int coord_system;    /* 0 Cartesian, 1 polar, 2 cylindrical, 3 spherical      */
  int comps;           /* components C of the state                             */
  int n_lap;           /* components solved                                     */
  int lap_comp[16];    /* their indices in the state                            */
  int elem_bytes;      /* 4 or 8: state, tables and coefficients                */
  int batch;           /* instances, at most PRML_JACOBI_MAX_BATCH              */
  int pitch;           /* state row pitch (elements)                            */
  int face_len;        /* boundary table entries per (face, component)          */
  int face_base;       /* table face = 2 * axis + side - face_base              */
  long long cstride;   /* state elements between component planes               */
  long long inst;      /* state elements between instances                      */
  unsigned long long dir_mask; /* bit (table face * C + comp): Dirichlet values */
  unsigned long long neu_mask; /* same for Neumann values                       */
  const void* dirichlet; /* (faces, C, face_len), NaN = free (state type)       */
  const void* neumann;
  /* Per-axis constants and per-vertex coefficient tables (state type):
   * inv_dxx[a] = 1 / dx_a^2 and two_dx[a] = 2 dx_a per kernel axis;
   * Cartesian: coef = {1 / sum_a 2 / dx_a^2};
   * polar / cylindrical (r along axis first_axis, n_r vertices):
   *   coef = [1 / (2 dx_r r)] [1 / r^2] [1 / denominator(r)], n_r each;
   * spherical (r along axis 0, phi along axis 2):
   *   coef = [1 / (dx_r r)] [1 / r^2] (n_r each) [cos phi] [1 / (2 dx_phi sin phi)]
   *   (n_phi each) [1 / (r^2 sin^2 phi)] [1 / denominator(r, phi)] (n_r x n_phi each). */
  double inv_dxx[3];
  double two_dx[3];
  const void* coef;
  double tol;
  long long max_iterations;
} prml_jacobi_params;

#define PRML_JACOBI_MAX_BATCH 64
/* sizeof(prml_jacobi_params), so bindings can check their mirror of it. */
int prml_jacobi_params_size(void);
/* Device scratch bytes prml_anti_laplacian needs for these parameters. */
long long prml_jacobi_scratch_bytes(const prml_jacobi_params* p);
/* On entry the solved components' planes of `state` hold the right-hand
 * side (the Laplacian); on return they hold the solution.  y_init: float64
 * [batch][*vertices][n_lap] (C order, the reference's random estimate).
 * `iterations` (host, may be NULL) receives each instance's iteration count.
 * Synchronises the stream.  PRML_ERR_CONVERGENCE if an instance is still
 * above tol after max_iterations. */
int prml_anti_laplacian(const prml_jacobi_params* p, void* state, const double* y_init, void* scratch,
                        long long scratch_bytes, long long* iterations, void* stream);

/* ---- implicit integrators (secant) ------------------------------------
 * Replace BackwardEulerMethod / CrankNicolsonMethod.integral and
 * ImplicitMethod._solve (pararealml/operators/fdm/numerical_integrator.py:
 * 135-270), whose scipy.optimize.newton call runs the element-wise secant
 * method on the whole state.  The caller evaluates the right-hand sides with
 * prml_fdm_rhs and drives the iteration:
 *   predict -> residual(p) -> residual(p1) -> { update -> stop(p, p1) ->
 *   swap (p, p1) -> [at max_iterations: stop(p, p1, force), end] ->
 *   swap (q0, q1) -> residual(p1) }, any number of iterations between two
 *   reads of the `finished` counters (finished instances are left alone),
 *   then finish on the stop results.
 * States are float64 in the planar layout [instance][C][rows][pitch].
 * counters: int [batch][4] = {residuals changed, some step >= tol,
 * no residual changed (stopped at the midpoint), instance finished}; an
 * instance whose `finished` entry is set is left unchanged by every call. */
typedef struct prml_implicit_params {
  int n[3];            /* vertices per kernel axis (1 where the mesh has none)  */
  int first_axis;      /* 3 - mesh dimension                                    */
  int comps;           /* components C                                          */
  int batch;
  int pitch;
  int face_len;        /* boundary table entries per (face, component)          */
  int face_base;       /* table face = 2 * axis + side - face_base              */
  int crank_nicolson;  /* 0: backward Euler, 1: Crank-Nicolson                  */
  long long cstride;   /* elements between component planes                     */
  long long inst;      /* elements between instances                            */
  unsigned long long d_mask;   /* bit c: component c has LHS.D_Y_OVER_D_T       */
  unsigned long long dir_mask; /* bit (table face * C + comp): Dirichlet values */
  const double* dirichlet;     /* (faces, C, face_len) at t + dt, NaN = free    */
  double dt;
  double a;            /* weight of the implicit term (backward Euler: 1)       */
  double tol;          /* secant tolerance on |step|                            */
  double dx;           /* offset of the second secant point: the float64 value
                        * of numpy's np.finfo(float).eps ** 0.33            */
} prml_implicit_params;

/* sizeof(prml_implicit_params), so bindings can check their mirror of it. */
int prml_implicit_params_size(void);
/* fu = dt f (dy/dt rows, 0 elsewhere); p = c(y + fu); p1 = the secant's
 * second point p (1 + dx) +- dx; flags reset (every element failing and
 * active). */
int prml_implicit_predict(const prml_implicit_params* p, const double* y, const double* f, double* fu, double* x0,
                          double* x1, unsigned char* flags, int* counters, void* stream);
/* q = x - c(y + (a dt) f + (1 - a) fu) (backward Euler: x - c(y + dt f)),
 * f = the right-hand sides at (t + dt, x); if q_prev is not NULL, counter 0
 * of an instance is set where q != q_prev. */
int prml_implicit_residual(const prml_implicit_params* p, const double* x, const double* y, const double* f,
                           const double* fu, double* q, const double* q_prev, int* counters, void* stream);
/* One secant step of every unfinished instance: x0 <- x1 - q1 (x1 - x0) /
 * (q1 - q0) where q1 != q0, midpoints where they are equal (once per
 * element), or all midpoints when no residual changed (counter 2). */
int prml_implicit_update(const prml_implicit_params* p, double* x0, const double* x1, const double* q0,
                         const double* q1, unsigned char* flags, int* counters, void* stream);
/* Per instance (out: double [batch][4]): failing elements, elements, failing
 * elements whose last residuals were equal, sum of (x1 - x0)^2 over those of
 * them that moved (the reference's warning and error conditions). */
int prml_implicit_status(const prml_implicit_params* p, const double* x0, const double* x1,
                         const unsigned char* flags, double* out, void* stream);
/* The end of a secant iteration (after update): the device iteration
 * counter `iteration` (int, zeroed by the caller at the step start)
 * advances to this iteration's number it (a forced stop keeps it); every
 * unfinished instance that stops now (no element stepped by tol or more, no
 * residual changed, or `force`) gets res = xs, its status sums as
 * prml_implicit_status computes them over (x0 = xs, x1 = xo) added to stats
 * (double [batch][4], zeroed at the step start), iterations[b] = it and its
 * `finished` counter set; then the other counters of every instance are
 * cleared for the next iteration.  Stopping after an update, xs is the new
 * iterate and xo the previous one (the reference returns the new iterate);
 * at the iteration limit, after the swap, xs is the previous iterate.  No
 * argument changes from one iteration to the next but the roles of the
 * buffers, which repeat every two iterations, so two iterations can be
 * recorded once as a CUDA graph and replayed. */
int prml_implicit_stop(const prml_implicit_params* p, const double* xs, const double* xo,
                       const unsigned char* flags, int* counters, int* iteration, int force, double* res,
                       double* stats, int* iterations, void* stream);
/* out = x on dy/dt rows, c(f) on the other rows (f: right-hand sides at the
 * step start; LHS.Y values, and LHS.Y_LAPLACIAN right-hand sides for the
 * Jacobi solve that follows). */
int prml_implicit_finish(const prml_implicit_params* p, const double* x, const double* f, double* out,
                         void* stream);

/* ---- layout conversion at the boundary ---------------------------------
 * The reference's state is a C-contiguous float64 array (*vertices, C)
 * (fdm_operator.py:53, solution.py:30-83); the kernels use planar padded
 * rows [instance][C][nx][pitch] in the state type.  src/dst strides are
 * the element distances between instances.  comp != 0 selects the
 * compensated float32 state: planes [C, 2C) hold the rounding remainder,
 * so the value is plane c + plane C + c (about 48 significant bits). */
int prml_pack(const double* src, void* dst, int elem_bytes, int batch, int comps, int nx, int ny,
              int pitch, long long src_bstride, long long dst_bstride, int comp, void* stream);
int prml_unpack(const void* src, int elem_bytes, double* dst, int batch, int comps, int nx, int ny,
                int pitch, long long src_bstride, long long dst_bstride, int comp, void* stream);

/* Gaussian initial states of a batch of instances on one mesh, float64
 * (batch, nv, comps) channel-last: replaces the host evaluation of
 * GaussianInitialCondition (pararealml/initial_condition.py:246-307,
 * multivariate_normal.pdf at the Cartesian images of the vertices, times the
 * multipliers).  x: (nv, dim) Cartesian vertex coordinates, dim <= 3;
 * params: per (instance, component) [mean (dim), U (dim x dim, row-major),
 * c0, multiplier], where U and c0 = rank log(2 pi) + log pdet come from the
 * covariance's eigendecomposition (scipy's pseudo-inverse square root).
 * The caller applies the mesh's Dirichlet vertex constraints after. */
int prml_gaussian_states(const double* x, long long nv, int dim, const double* params, int batch, int comps,
                         double* out, void* stream);

/* ---- Parareal correction (FP64) ---------------------------------------
 * Replaces the MPI Allgather of corrections and the sequential coarse
 * sweep of PararealOperator.solve (parareal_operator.py:152-188) and its
 * termination norm (_should_terminate, :53-100). */
/* `comp` (here and below): 0 for plain states, else the number of float64
 * elements per instance, for compensated states (per instance: comp "hi"
 * words, then comp "lo" words). */
int prml_pr_cast(const double* src, void* dst, int elem_bytes, long long n, long long comp,
                 void* stream);
/* corr = fine_end - coarse_old (parareal_operator.py:164) */
int prml_pr_correct(const void* fine_end, int elem_bytes, const double* coarse_old, double* corr,
                    long long n, long long per_instance, const int* active, int batch,
                    long long comp, void* stream);
/* coarse_store = coarse_new (if not NULL); u_next = coarse_store + corr;
 * u_next_state = u_next in the state type (if not NULL) (:179-185) */
int prml_pr_advance(const void* coarse_new, int elem_bytes, double* coarse_store,
                    const double* corr, double* u_next, void* u_next_state, long long n,
                    long long per_instance, const int* active, int batch, long long comp,
                    void* stream);
/* dst = src where the instance is active (keeps each instance's border
 * points from the start of its last iteration, for the final fine sweep). */
int prml_pr_copy(const double* src, double* dst, long long n, long long per_instance,
                 const int* active, int batch, void* stream);
/* delta = u_end - end_state: the constant offset the reference adds to each
 * slice's fine trajectory in the final assembly (parareal_operator.py:192). */
int prml_pr_end_delta(const double* u_end, const void* end_state, int elem_bytes, double* delta,
                      long long n, long long comp, void* stream);
/* Scratch elements (doubles) prml_pr_update_norm needs for `partial`. */
long long prml_pr_norm_scratch_elems(int slices, int batch, int comps, int chunks);
/* out[b*comps + c] = max_j sqrt(mean((new_j - old_j)^2)) per instance and
 * component (parareal_operator.py:85-100); like np.maximum there, a NaN
 * RMS of any slice makes the result NaN. */
int prml_pr_update_norm(const double* new_pts, const double* old_pts, int slices, int batch,
                        int comps, int nx, int ny, int pitch, int chunks, double* partial,
                        double* out, void* stream);

/* ---- learned coarse operator: residual CNN ----------------------------
 * Replaces the model of the reference's SupervisedMLOperator
 * (pararealml/operators/ml/supervised/supervised_ml_operator.py:16-128,
 * sklearn/keras regressors trained on oracle trajectories) with
 *   y = u + s_out * conv(relu(conv(... relu(conv(s_in * u)))))
 * six 3x3 "same" convolutions 2 -> 32 -> 32 x4 -> 2.  States u, y are planar
 * [B][2][H][pitch] (elem_bytes 4 or 8); hidden activations and gradients are
 * bf16 NHWC [B][H][W][32]; weights fp32 [9][ci][co] (taps t = (dy+1)*3 +
 * (dx+1)); the 32 -> 32 layers take bf16 copies packed by
 * prml_cnn_pack_mid: forward [9][co][ci], dgrad [9][ci][co] with flipped
 * taps.  `parts` is the number of CTAs (and partial sums) of a reduction;
 * `scratch` is caller memory of the size the *_scratch_elems functions give. */
int prml_cnn_in_fwd(const void* u, int elem_bytes, int pitch, const float* w0, const float* b0,
                    const float* s_in, void* x1, int B, int H, int W, void* stream);
int prml_cnn_mid_fwd(const void* x, const void* wf, const float* bias, void* y, int B, int H, int W,
                     void* stream);
int prml_cnn_out_fwd(const void* x5, const float* w5, const float* b5, const float* s_out,
                     const void* u, void* y, int elem_bytes, int pitch, int B, int H, int W,
                     void* stream);
/* dy: fp32 dense [B][2][H][W] gradient of the loss w.r.t. y */
int prml_cnn_out_bwd(const float* dy, const void* x5, const float* w5, const float* s_out, void* dx5,
                     float* dw5, float* db5, int parts, float* scratch, int B, int H, int W,
                     void* stream);
int prml_cnn_mid_dgrad(const void* g, const void* wd, const void* mask, void* gx, int B, int H, int W,
                       void* stream);
long long prml_cnn_wgrad_scratch_elems(int parts);
int prml_cnn_mid_wgrad(const void* x, const void* g, float* dw, float* db, int parts, float* scratch,
                       int B, int H, int W, void* stream);
long long prml_cnn_thin_scratch_elems(int parts);
int prml_cnn_in_wgrad(const void* g1, const void* u, int elem_bytes, int pitch, const float* s_in,
                      float* dw0, float* db0, int parts, float* scratch, int B, int H, int W,
                      void* stream);
/* dy = 2 (y - target) / n, partial[k] = sums of squared errors of CTA k */
int prml_cnn_mse(const void* y, const void* target, int elem_bytes, int pitch, int B, int H, int W,
                 float* dy, double* partial, int parts, void* stream);
int prml_cnn_adam(float* params, const float* grads, float* m, float* v, long long n, float lr,
                  float beta1, float beta2, float eps, int step, void* stream);
int prml_cnn_pack_mid(const float* w, void* wf, void* wd, void* stream);
/* Selects the kernel behind prml_cnn_mid_fwd / prml_cnn_mid_dgrad: 1 (the
 * default) the tcgen05 implicit GEMM with TMEM accumulators, 0 the mma.sync
 * one.  Returns the previous setting.  No reference counterpart. */
int prml_cnn_set_tensor_path(int tcgen05);
/* Synchronising check of the tcgen05 convolution's device status flag
 * (set when a bounded pipeline wait timed out); clears it and returns
 * PRML_ERR_CUDA if it was set. */
int prml_cnn_status(void);

/* ---- device rate probe -------------------------------------------------
 * No counterpart in the reference.  Measures the float64 fused multiply-add
 * rate of the current device (multiply-adds per second, best of three
 * event-timed launches on `stream`, which it synchronises): the compute
 * roofline of the float64 stencil kernels, which this GPU's small float64
 * pipe bounds. */
int prml_measure_fp64_fma(double* fma_per_s, void* stream);

/* ---- allocation-free variant ------------------------------------------
 * No counterpart in the reference.  Same result as prml_pr_update_norm, but
 * the partial sums go to a fixed array inside the library instead of a
 * caller buffer, so the call allocates nothing and needs no scratch from the
 * caller.  It is for callers that cannot allocate device memory where they
 * need the norm: a host application that hands this library only the
 * buffers it owns (a plain ctypes or cgo binding with no device allocator of
 * its own), or one that plans every allocation up front and forbids new ones
 * while a run is in progress.
 *   - Limit: slices * batch * comps * chunks <= PRML_NOALLOC_NORM_SCRATCH_ELEMS
 *     doubles (2 MiB); larger requests return PRML_ERR_ARG.
 *   - Every GPU that loads the library holds the array until the process
 *     exits.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.  The address is kept with the context it
 *     was found in; after a device reset (a new context) the next call looks
 *     it up again, so that call too belongs before any capture.
 *   - All calls on a device share the array: calls that overlap on the GPU
 *     (e.g. on two streams at once) race.  Nothing in it needs to start at
 *     zero: each call writes every slot it reads. */
#define PRML_NOALLOC_NORM_SCRATCH_ELEMS 262144
#define PRML_NOALLOC_MAX_DEVICES 64
int prml_pr_update_norm_noalloc(const double* new_pts, const double* old_pts, int slices,
                                int batch, int comps, int nx, int ny, int pitch, int chunks,
                                double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PARAREALML_GB300_H */
