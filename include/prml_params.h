/*
 * Launch parameter block shared by the host runtime (prml_core.cpp) and the
 * generated stencil kernels (fdm_step.cuh, compiled at run time by NVRTC).
 *
 * Plain C, fixed-width fields only, so that the host and the device agree on
 * the layout without any C++ or torch types crossing the boundary.
 *
 * State layout in device memory: [instance][component][row][pitch] with the
 * last mesh axis contiguous (kernel axis 1 = "cols", extent ny) and the
 * first mesh axis strided by `pitch` (kernel axis 0 = "rows", extent nx).
 * A 1D mesh of n vertices is stored as nx = 1, ny = n; an ODE as nx = ny = 1.
 *
 * The step kernels read their input through a 5D TMA tensor map over
 * [slot][instance][C][row][col] (dims listed innermost first when encoded),
 * passed as a second, __grid_constant__ kernel parameter; `in` is kept for
 * reference and `in_slot` selects the slot.
 */
#ifndef PRML_PARAMS_H
#define PRML_PARAMS_H

#ifdef __cplusplus
extern "C" {
#endif

/* Most time steps one launch of a temporally blocked step kernel takes. */
#define PRML_TB_MAX 8

typedef struct prml_step_params {
  const void* in;          /* state at the start of the step            */
  void* out;               /* state at the end of the step              */
  long long in_bstride;    /* elements between instances in `in`        */
  long long out_bstride;   /* elements between instances in `out`       */
  long long cstride;       /* elements between components (nx * pitch)  */
  int pitch;               /* row pitch in elements                     */
  int nx, ny;              /* vertices along kernel axes 0 and 1        */
  int batch;               /* number of instances                       */
  int face_len;            /* entries per face row of the BC tables     */
  int elem_bytes;           /* bytes per state element: 4 or 8         */
  double t;                /* time at the start of the step             */
  double dt;               /* step size                                 */
  const double* t_offset;  /* per-instance time offset, may be NULL     */
  const void* dirichlet;   /* [4 faces][C][face_len], NaN = free        */
  const void* neumann;     /* [4 faces][C][face_len], NaN = free        */
  const double* coord0;    /* vertex coordinates along kernel axis 0    */
  const double* coord1;    /* vertex coordinates along kernel axis 1    */
  /* derived mesh constants (host computes them once per plan)          */
  double inv_2dx0, inv_2dx1; /* 1 / (2 dx)                              */
  double inv_dxx0, inv_dxx1; /* 1 / (dx * dx)                           */
  double two_dx0, two_dx1;   /* 2 dx (Neumann ghost offset)             */
  int in_slot;             /* slot coordinate of `in` in its tensor map */
  int max_ctas;            /* cap on the persistent grid, 0 = fill the GPU */
  int* status;             /* device flag set to 1 when a bounded wait
                              inside a kernel times out (may be NULL)    */
  /* temporal blocking: a kernel built for tb_max > 1 takes tb_steps time
   * steps per launch on one staged tile (halo tb_max vertices); step j of
   * the launch (j < tb_steps - 1) is stored to tb_out[j] when that is not
   * NULL, the last step to `out`.  The host runtime fills these per launch. */
  int tb_max;              /* steps the kernel can take per launch (>= 1) */
  int tb_steps;            /* steps this launch takes, 1..tb_max          */
  long long tb_bstride;    /* elements between instances in tb_out states */
  void* tb_out[PRML_TB_MAX - 1];
  /* float32 copies of the step size, the mesh constants and the vertex
   * coordinates: float32 kernels read these and so run no double-precision
   * arithmetic (a slow pipe on GB300) outside time-dependent right-hand
   * sides.  The host rounds each double to nearest, as a device cast would. */
  float dt_f;
  float inv_2dx0_f, inv_2dx1_f, inv_dxx0_f, inv_dxx1_f, two_dx0_f, two_dx1_f;
  const float* coord0_f;
  const float* coord1_f;
  /* time-dependent boundary conditions: `dirichlet` / `neumann` hold one
   * table per half step of the run (time t0 + k dt / 2 for table k),
   * bc_stride elements apart; bc_slot0 is the table of the launch's first
   * step start (the host runtime sets it).  0 for static conditions. */
  long long bc_stride;
  int bc_slot0;
  /* 3D meshes (kernel axes 0 = planes, 1 = rows, 2 = columns): nx rows
   * and ny columns per plane as above, nz planes (1 for 0/1/2-D), planes
   * nx * pitch elements apart; a 3D kernel's tile depth and TMA box depth */
  int nz;
  int tile_z;
  int box_planes;
  double inv_2dx2, inv_dxx2, two_dx2;
  float inv_2dx2_f, inv_dxx2_f, two_dx2_f;
  int pad3;
  const double* coord2;
  const float* coord2_f;
  /* dx^2 per kernel axis (2D: axes 0, 1; 3D: the planes' axis in dxx2):
   * divisors of the second differences of modules generated with exact
   * division (float64 right-hand sides of the implicit integrators, which
   * round like the reference's numpy expressions) */
  double dxx0, dxx1, dxx2;
  /* Bound of every wait of the step kernels (TMA staging), in ns of
   * %globaltimer; 0 = 2 s.  After a wait gives up the CTA sets *status,
   * drains its own copies (bounded) and returns. */
  unsigned long long wait_limit_ns;
  /* Tests of that error path only: 1 = arm the staging barriers without
   * issuing the copies, so that every wait runs out after wait_limit_ns
   * and nothing else happens (2: the multi-round kernel waits for one
   * grid-barrier arrival more than the grid has).  0 in every solve. */
  int wait_probe;
  int pad4;
  /* Per-instance offset (in half-step tables) added to bc_slot0, or NULL:
   * a batch whose instances start at different times of one set of
   * time-dependent boundary tables (Parareal slices). */
  const int* bc_inst_slot;
} prml_step_params;

/* ---- multi-round launches ------------------------------------------------
 * One persistent cooperative launch takes every step of up to
 * PRML_MULTI_MAX_GROUPS groups of instances (each group: one mesh, its own
 * time step and step count), round by round: round r is step r of every
 * group that has more than r steps, its tiles spread over the whole grid,
 * and the rounds are separated by a grid-wide barrier. */
#define PRML_MULTI_MAX_GROUPS 8

typedef struct prml_multi_group {
  prml_step_params p;    /* geometry, tables and constants of the group; `in`,
                            `out`, `t`, `in_slot` and `bc_slot0` are set per
                            round on the device.  in_bstride = out_bstride:
                            `first` and `main` share the instance stride.     */
  const void* first;     /* state the group's first step reads               */
  void* main;            /* slotted buffer the group's steps write           */
  long long slot_stride; /* elements between slots of `main`                 */
  double t0;             /* time at the start of the first step              */
  int n_steps;           /* the group takes part in rounds 0 .. n_steps - 1  */
  int ping_pong;         /* 0: step s goes to slot s (a full trajectory);
                            1: to slot s % 2 (the final state only)          */
  int tiles_x;           /* tiles per instance along columns (host fills)    */
  int tiles_y;           /* tiles per instance along rows (host fills)       */
} prml_multi_group;

typedef struct prml_multi_params {
  const prml_multi_group* groups; /* device array of n_groups descriptors      */
  const void* maps;      /* device array of 2 n_groups tensor maps (128 bytes
                            each, 64-byte aligned): 2g over `first`, 2g + 1
                            over `main`                                       */
  unsigned long long* barrier; /* arrival counter, zero at launch            */
  int* status;           /* set to 1 when a bounded wait times out           */
  int n_groups;
  int n_rounds;          /* largest n_steps of the groups                    */
} prml_multi_params;

#ifdef __cplusplus
}
#endif

#endif /* PRML_PARAMS_H */
