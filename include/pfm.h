/*
 * pfm.h -- C ABI of libpfm.so, the sm_103a (GB300) implementation of the particle-flow-map time
 * step of the impulse-based Eulerian-Lagrangian fluid solver (zjw49246/particle-flow-maps).
 *
 * Every entry point replaces one Taichi kernel (or kernel group) that the reference's step loop
 * calls; each declaration cites the reference interface it replaces (path:line within the
 * reference project).  Conventions:
 *
 *  - All array arguments are caller-owned DEVICE pointers (e.g. torch tensor data_ptr()).
 *  - Grid fields are f32, C-order with the last index fastest, face grids padded by one along
 *    their own axis: u_x [nx+1][ny][nz], u_y [nx][ny+1][nz], u_z [nx][ny][nz+1]
 *    (2D: u_x [nx+1][ny], u_y [nx][ny+1]); cell fields [nx][ny][nz].
 *  - Particle fields are structure-of-arrays: a field of n-vectors is n contiguous runs of P
 *    floats ([n][P]).  A per-particle set of d vectors of size d (T_x/T_y/T_z, init_C_x/..)
 *    is [d][d][P]: vector v, component c of particle q sits at (v*d + c)*P + q.
 *    (The reference's Taichi layout is AoS [P][n]; the Python layer converts for the oracle.)
 *  - Every call takes the CUDA stream to run on (cudaStream_t passed as void*) and is
 *    asynchronous, except where a function is documented as a synchronization point because it
 *    returns a host value.
 *  - Every function returns a pfm_status; pfm_last_error() gives the message of the last error
 *    on that handle.  A handle is used by one host thread at a time.
 */
#ifndef PFM_H_
#define PFM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pfm_status {
  PFM_OK = 0,
  PFM_ERR_NULL = 1,           /* a required pointer is NULL */
  PFM_ERR_SHAPE = 2,          /* configuration / size mismatch */
  PFM_ERR_WORKSPACE = 3,      /* no workspace bound, or too small */
  PFM_ERR_NOT_CONVERGED = 4,  /* MGPCG reached max_iters (results are still written) */
  PFM_ERR_NONFINITE = 5,      /* NaN/Inf met in a reduction */
  PFM_ERR_CUDA = 6,           /* a CUDA runtime call failed */
  PFM_ERR_ARG = 7             /* an argument is out of range */
} pfm_status;

/* Solver configuration.  Mirrors MGPCG_3(boundary_types, N, base_level) (3D/mgpcg.py:350-357,
 * 17-60) and the step constants of hyperparameters.py. */
typedef struct pfm_config {
  int dim;                   /* 2 or 3 */
  int res[3];                /* res_x, res_y, res_z (res_z ignored in 2D) */
  double dx;                 /* cell size; the reference uses dx = 1/res_y (3D/run_3D.py:16) */
  int64_t particles;         /* particle count P */
  int base_level;            /* level formula int(log2(min N)) - base_level + 1 (3D/mgpcg.py:28) */
  int mg_levels;             /* > 0 overrides the formula */
  int pre_post_smoothing;    /* 2 (3D/mgpcg.py:29) */
  int bottom_smoothing;      /* 50 (3D/mgpcg.py:30) */
  int boundary[3][2];        /* 1 = Dirichlet, 2 = Neumann, per axis low/high (3D/run_3D.py:28) */
  int use_apic;              /* hyperparameters.use_APIC */
} pfm_config;

typedef struct pfm_handle pfm_handle;

/* Options and statistics of one MGPCG solve: MGPCG.solve(max_iters, eps, tol)
 * (3D/mgpcg.py:202-280).  tol_mode 0 stops when r.r < tol (the reference's absolute rule);
 * tol_mode 1 stops when sqrt(r.r / r0.r0) < tol (relative to the first residual); tol_mode 2
 * stops when sqrt(r.r / b.b) < tol (relative to the recentred right-hand side b; the same as mode
 * 1 for a zero initial guess, and the rule to compare warm-started solves at equal residual).
 *
 * precision 0 is the reference's FP32 solve.  precision 1 / 2 is the mixed form: the multigrid
 * levels (the V-cycle's z and r on every level) are stored in FP16 / BF16 and smoothed,
 * restricted and prolonged with FP32 arithmetic; the PCG vectors x, r, p, Ap stay FP32; inner
 * products and norms are compensated FP32 sums per thread combined in FP64.
 * warm_start 1 starts from the caller's current pressure (p_out of pfm3/pfm2_poisson, x_out of
 * pfm_mgpcg_solve) instead of zero; warm_start 2 starts from the linear extrapolation
 * 2 p - p_before of that pressure and what the same buffer held at the start of its previous solve
 * (in a step loop: the solution before it), and warm_start 3 from the quadratic extrapolation
 * 3 (p - p_before) + p_before2 through the last three.  The handle keeps the two earlier values in
 * its workspace for up to two buffers (their pointers name the slots; a third buffer is
 * PFM_ERR_ARG); with fewer kept (a new history) the solve starts from the highest order they allow
 * (p alone, then the linear form).
 * true_residual_every K > 0 recomputes the true residual |b - A x| every K iterations and after
 * the last one and reports it (stats.rTr_true); the stopping rule stays the reference's, on the
 * recursive residual (x is stored in f32, whose rounding alone leaves a true residual of about
 * 2e-5 relative at 64^3, above a 1e-6 rule).  With true_residual_replace (mixed solves) x is kept
 * in FP64 during the solve, and every K iterations, and whenever the recursive residual passes
 * the rule, b - A x is formed in FP64, replaces the recursive residual and decides convergence:
 * the solve stops on its true residual; the caller receives x rounded to f32. */
typedef struct pfm_solve_opts {
  int max_iters;   /* 400 in Poisson() (3D/mgpcg.py:422); -1 = unlimited */
  double eps;      /* 1e-12, added to the denominators of alpha and beta */
  double tol;      /* 1e-12 in Poisson() */
  int tol_mode;    /* 0 absolute r.r, 1 relative to r0, 2 relative to b */
  int check_every; /* the iteration loop runs on the device (a CUDA graph WHILE node) and the
                      host waits once per solve; with max_iters = -1 the host relaunches the
                      loop every check_every iterations (>= 1) until it converges */
  int precision;   /* 0 FP32 (reference), 1 FP16 multigrid levels, 2 BF16 multigrid levels */
  int warm_start;  /* 1: initial guess = the caller's pressure buffer; 2 / 3: its linear /
                      quadratic extrapolation through the buffer's last solutions */
  int true_residual_every; /* 0: never (reference); K > 0: check every K iterations and at the end */
  int true_residual_replace; /* mixed solve with K > 0: 1 = x accumulates in FP64 and the true residual
                                b - A x (FP64) replaces the recursive one every K iterations and before
                                convergence is accepted; 0 = the check only reports */
} pfm_solve_opts;

typedef struct pfm_solve_stats {
  int iterations;      /* the `it` the reference prints on convergence */
  int converged;       /* 1 if the stopping rule was met */
  double rTr;          /* final r.r (the true residual when true_residual_every > 0) */
  double rTr0;         /* r.r of the initial residual */
  double bTb;          /* b.b of the recentred right-hand side */
  double rTr_true;     /* |b - A x|^2 after the solve (true_residual_every > 0), else -1 */
} pfm_solve_stats;

/* ---- handle, workspace, errors ------------------------------------------------------------- */

/* Creates a handle for one scene.  No device memory is allocated by the library.  Grids whose
 * cell or face fields hold 2^31 or more entries are rejected (PFM_ERR_SHAPE): the grid kernels
 * index with 32-bit integers. */
int pfm_create(const pfm_config* cfg, pfm_handle** out);
int pfm_destroy(pfm_handle* h);
/* Bytes of device scratch the handle needs (sort buffers, P2G payload, MGPCG hierarchy). */
int pfm_workspace_size(const pfm_handle* h, size_t* bytes);
/* Binds caller-allocated device scratch (>= pfm_workspace_size bytes, 256-byte aligned). */
int pfm_set_workspace(pfm_handle* h, void* dptr, size_t bytes);
const char* pfm_last_error(const pfm_handle* h);
const char* pfm_status_string(int status);
/* Number of MGPCG levels the handle uses. */
int pfm_mg_levels(const pfm_handle* h, int* levels);
/* Number of kernels launched through this handle since pfm_create (bookkeeping for benchmarks). */
int pfm_launch_count(const pfm_handle* h, uint64_t* launches);
/* FP32 roofline denominator: times `reps` launches of an FMA-throughput kernel (8 independent
 * chains per thread, `blocks_per_sm` x SMs blocks of 256 threads, `iters` iterations; packed = 1
 * advances them as 4 pairs with packed f32x2 FMAs) on `stream` with CUDA events and writes the
 * best rate in TFLOP/s (2 flops per FMA).  `sink` is one device float the kernel may write (it
 * does not, for any result the chains reach).  Synchronous. */
int pfm_measure_fp32_peak(float* sink, int blocks_per_sm, int iters, int reps, int packed, double* tflops,
                          void* stream);

/* Launch-shape tunables of a handle.  Every value gives the same results bit for bit (the sums keep
 * their order); they only change how the work maps to the GPU.  Setting one drops the handle's
 * captured graphs (they are rebuilt on next use); a batch that holds the handle must be rebuilt
 * (a new pfm_batch).  pfm.tune.autotune picks them by timing on a scene's own data. */
#define PFM_TUNE_P2G2_COLUMN 1    /* faces per thread of the 2D P2G column gather, 1..64 (8) */
#define PFM_TUNE_MG_TAIL_CELLS 2  /* MGPCG levels with at most this many cells run the rest of the
                                     V-cycle in one thread block; 0 = none (4096) */
#define PFM_TUNE_SMOOTH_TMA 3     /* 1: 3D 16-bit MGPCG levels are smoothed from tiles the TMA stages
                                     in shared memory; 0: from global memory (0) */
#define PFM_TUNE_CUBE_KERNELS 4   /* 1: on cubic 64^3, 128^3, 256^3 and 512^3 grids the 3D RK4 and
                                     midpoint kernels run instances compiled for that extent (the
                                     face-field strides are constants); 0: strides read at run time (1) */
#define PFM_TUNE_MIDPOINT_CENTRE 5 /* 1: the 3D midpoint's first RK stage, which samples the face centre,
                                     uses its constant weights and leaves out the zero-weight taps
                                     (interior faces, power-of-two dx); 0: the generic taps (1) */
int pfm_set_tuning(pfm_handle* h, int key, int value);
int pfm_get_tuning(const pfm_handle* h, int key, int* value);

/* ---- 3D step phases ------------------------------------------------------------------------ */

/* calc_max_speed (3D/run_3D.py:95-103): max over cells of the centre-averaged speed, floor 1e-3.
 * Writes the f32 result to *max_dev (device pointer).  Asynchronous. */
int pfm3_calc_max_speed(pfm_handle* h, const float* u_x, const float* u_y, const float* u_z,
                        float* max_dev, void* stream);

/* init_particles_imp / init_particles_imp_grad_m (3D/init_conditions.py:254-273): G2P of the
 * grid velocity (imp_out [3][P], may be NULL) and its gradient (C_out [3][3][P] = init_C_x/y/z,
 * may be NULL) at the particle positions pos [3][P]. */
int pfm3_g2p(pfm_handle* h, const float* pos, const float* u_x, const float* u_y, const float* u_z,
             float* imp_out, float* C_out, void* stream);

/* update_T (3D/run_3D.py:430-439): T_init <- cols(T_gm) @ cols(T_init); then, when reset_gm is
 * nonzero, reset_T_to_identity(T_gm) (3D/run_3D.py:133-140).  Both [3][3][P]. */
int pfm3_update_T(pfm_handle* h, float* T_init, float* T_gm, int reset_gm, void* stream);

/* reset_T_to_identity (3D/run_3D.py:133-140) on a [3][3][P] field. */
int pfm3_reset_T(pfm_handle* h, float* T, void* stream);

/* RK4_T_forward (3D/run_3D.py:175-219): forward RK4 of positions pos [3][P] and of the three
 * rows of T [3][3][P] (dT/dt = -(grad u)^T T) in the velocity field u over dt.  In place. */
int pfm3_rk4_T_forward(pfm_handle* h, float* pos, float* T, const float* u_x, const float* u_y,
                       const float* u_z, float dt, void* stream);

/* Midpoint velocity (3D/run_3D.py:779-788 before the projection): reset_to_identity_grid,
 * RK4_grid over -dt_half for every face family, then advect_u: u1 = T . u0(psi).
 * u0 and u1 must not alias.  psi_out/T_out ([F][3] per family, AoS like the reference grids)
 * may be NULL; when given they receive psi_{x,y,z}_grid / T_{x,y,z}_grid. */
int pfm3_midpoint(pfm_handle* h, const float* u0_x, const float* u0_y, const float* u0_z,
                  float* u1_x, float* u1_y, float* u1_z, float dt_half, float* psi_out[3],
                  float* T_out[3], void* stream);

/* get_particles_id_in_every_cell (3D/run_3D.py:342-351) as a deterministic counting sort: bins
 * the particles by int(pos/dx) (clamped to the grid) and orders each bin by particle index.
 * Results stay in the workspace; cell_count (may be NULL, [C] int32) and order (may be NULL,
 * [P] int32, the stable permutation) are copied out when given. */
int pfm3_sort_particles(pfm_handle* h, const float* pos, int* cell_count, int* order, void* stream);

/* P2G (3D/run_3D.py:441-552): APIC transfer of impulse m = T_gm^T T_init^T-composed init_imp
 * with affine term (T_gm^T init_C T_gm) to the faces, normalised by the weight sums.
 * Deterministic, no float atomics: particles are counting-sorted into cell bins, each cell's
 * particles are summed into the window of faces they reach, and cell tiles merge the windows in
 * a fixed order.  Writes u_x/u_y/u_z and the weight grids w_x/w_y/w_z. */
int pfm3_p2g(pfm_handle* h, const float* init_imp, const float* pos, const float* T_gm,
             const float* T_init, const float* init_C, float* u_x, float* u_y, float* u_z,
             float* w_x, float* w_y, float* w_z, void* stream);

/* RK4_T_forward followed by P2G, the pair the step loop calls back to back (3D/run_3D.py:795-812).
 * pfm3_rk4_p2g_records advances pos/T_gm in the advecting velocity ua over dt (as
 * pfm3_rk4_T_forward) and, in the same kernel, writes each advected particle's P2G record and
 * cell key into the workspace, so the particle state is read once.  pfm3_p2g_from_records then
 * runs the rest of P2G (bin sort, cell tiles, normalisation) from those records; it fails with
 * PFM_ERR_ARG if no records are present (a sort or 2D P2G call on the handle in between
 * overwrites them).  pfm3_rk4_p2g does both.  Results are bitwise those of
 * pfm3_rk4_T_forward(pos, T_gm, ua, dt) followed by pfm3_p2g(init_imp, pos, T_gm, T_init,
 * init_C, u, w).  ua may be the same grids as u. */
int pfm3_rk4_p2g_records(pfm_handle* h, float* pos, float* T_gm, const float* ua_x,
                         const float* ua_y, const float* ua_z, float dt, const float* init_imp,
                         const float* T_init, const float* init_C, void* stream);
int pfm3_p2g_from_records(pfm_handle* h, float* u_x, float* u_y, float* u_z, float* w_x,
                          float* w_y, float* w_z, void* stream);

/* pfm3_rk4_p2g_records preceded by the flow-map gradient reinitialisation of the step
 * (3D/run_3D.py:768-772), in the same kernel: init_C <- grad u(pos) in the velocity u
 * (init_particles_imp_grad_m), T_init <- cols(T_gm) @ cols(T_init) (update_T), T_gm <- I, then
 * RK4 of pos/T_gm in ua over dt from the identity, and the P2G records.  Bitwise the same as
 * pfm3_g2p(pos, u, NULL, init_C), pfm3_update_T(T_init, T_gm, 1) and
 * pfm3_rk4_p2g_records(pos, T_gm, ua, dt, init_imp, T_init, init_C); the reinitialisation reads
 * the same pos as the RK4, so it may run after the midpoint solve. */
int pfm3_gradm_rk4_p2g_records(pfm_handle* h, float* pos, float* T_gm, float* T_init, float* init_C,
                               const float* init_imp, const float* u_x, const float* u_y,
                               const float* u_z, const float* ua_x, const float* ua_y,
                               const float* ua_z, float dt, void* stream);
int pfm3_rk4_p2g(pfm_handle* h, float* pos, float* T_gm, const float* ua_x, const float* ua_y,
                 const float* ua_z, float dt, const float* init_imp, const float* T_init,
                 const float* init_C, float* u_x, float* u_y, float* u_z, float* w_x, float* w_y,
                 float* w_z, void* stream);

/* MGPCG_3.Poisson (3D/mgpcg.py:425-430): apply_bc, divergence, MGPCG solve of the pressure,
 * subtract_grad_p, apply_bc.  In place on u.  p_out [nx][ny][nz] (may be NULL) receives the
 * pressure.  SYNCHRONIZATION POINT: returns after the solve finished; stats may be NULL. */
int pfm3_poisson(pfm_handle* h, float* u_x, float* u_y, float* u_z, float* p_out,
                 const pfm_solve_opts* opts, pfm_solve_stats* stats, void* stream);

/* ---- 2D step phases ------------------------------------------------------------------------ */

int pfm2_calc_max_speed(pfm_handle* h, const float* u_x, const float* u_y, float* max_dev,
                        void* stream); /* 2D/run_2D.py:101-108 */
/* init_particles_imp / _grad_m (2D/init_conditions.py:184-210): imp_out [2][P], C_out [2][2][P] */
int pfm2_g2p(pfm_handle* h, const float* pos, const float* u_x, const float* u_y, float* imp_out,
             float* C_out, void* stream);
/* RK4_T_forward (2D/run_2D.py:304-341), advect_psi as in the reference */
int pfm2_rk4_T_forward(pfm_handle* h, float* pos, float* T, const float* u_x, const float* u_y,
                       float dt, int advect_psi, void* stream);
/* update_particles_grad_m (2D/run_2D.py:526-536): C = T^T-sandwich of init_C */
int pfm2_update_grad_m(pfm_handle* h, float* C, const float* init_C, const float* T_gm, void* stream);
/* update_T (2D/run_2D.py:538-546): T = cols(T_gm) @ cols(T_init) */
int pfm2_update_T(pfm_handle* h, float* T, const float* T_init, const float* T_gm, void* stream);
/* update_particles_imp (2D/run_2D.py:517-524): imp = cols(T) @ init_imp */
int pfm2_update_imp(pfm_handle* h, float* imp, const float* init_imp, const float* T, void* stream);
/* reset_T_to_identity (2D/run_2D.py:141-146) */
int pfm2_reset_T(pfm_handle* h, float* T, void* stream);
/* midpoint (2D/run_2D.py:866-871 before the projection) */
int pfm2_midpoint(pfm_handle* h, const float* u0_x, const float* u0_y, float* u1_x, float* u1_y,
                  float dt_half, float* psi_out[2], float* T_out[2], void* stream);
int pfm2_sort_particles(pfm_handle* h, const float* pos, int* cell_count, int* order, void* stream);

/* Particle binning that allocates nothing (no counterpart in the reference, which sorts inside a
 * Taichi kernel on fields it allocated itself).  For callers that must not allocate device memory
 * at all: code running inside a host allocator's or framework's own memory callbacks, embedders
 * whose pools own every byte of the device, or anyone without a pfm_handle (pfm_create and the
 * workspace both allocate).  Same result as pfm3_sort_particles / pfm2_sort_particles, bit for
 * bit: cell_count [C] int32 (C = product of res[0..dim)) and order [P] int32, the stable
 * permutation by int(pos/dx) clamped to the grid.  pos [dim][P] f32.
 *
 * Scratch is one fixed array inside the library's device image, so the sizes are bounded:
 * particles <= PFM_NOALLOC_MAX_PARTICLES and C <= PFM_NOALLOC_MAX_CELLS, else PFM_ERR_SHAPE
 * (nothing launched).  Every call on a device shares that array and leaves its last contents
 * there; calls that overlap in time (two streams, two host threads) race on it and must be
 * serialised by the caller.  The first call on each device (that device current) looks up the
 * array's address; make that first call before any stream capture.  The address is kept for the
 * life of the process: after a cudaDeviceReset() of a device, do not call this on that device.
 * Returns PFM_ERR_ARG (dim not 2/3, dx <= 0, particles < 0), PFM_ERR_NULL, PFM_ERR_SHAPE or
 * PFM_ERR_CUDA (launch error). */
#define PFM_NOALLOC_MAX_PARTICLES (1 << 21)
#define PFM_NOALLOC_MAX_CELLS (1 << 18)
int pfm_sort_particles_noalloc(int dim, const int res[3], double dx, int64_t particles, const float* pos,
                               int* cell_count, int* order, void* stream);
/* P2G (2D/run_2D.py:548-611): impulse with APIC C [2][2][P] and the reference map psi [2][P]
 * (psi_x/psi_y grids [F][2] may be NULL). */
int pfm2_p2g(pfm_handle* h, const float* imp, const float* pos, const float* C, const float* psi,
             float* u_x, float* u_y, float* psi_x, float* psi_y, float* w_x, float* w_y, void* stream);
/* MGPCG_2.Poisson (2D/mgpcg.py:342-347). SYNCHRONIZATION POINT. */
int pfm2_poisson(pfm_handle* h, float* u_x, float* u_y, float* p_out, const pfm_solve_opts* opts,
                 pfm_solve_stats* stats, void* stream);

/* ---- the whole step as one CUDA graph --------------------------------------------------------
 * pfm3_step / pfm2_step run one iteration of the step loop (3D/run_3D.py:716-822,
 * 2D/run_2D.py:772-909) as a single CUDA graph launch on `stream`, with no host synchronization:
 * calc_max_speed, the frame clock (dt = CFL dx / max_speed clamped to the next frame, in double as
 * the reference's Python), the reinitialisation schedule, the midpoint velocity and its projection,
 * RK4 + P2G and the final projection all run on the device; the reinitialisations are IF nodes
 * and each MGPCG solve is a WHILE node, so a step does exactly the work of the eager phase calls
 * (pfm.Sim3D / Sim2D), bitwise.  The 3D step is the fused form (gradient reinitialisation + RK4
 * + P2G records in one kernel).  The graph is captured on the first call and rebuilt only when a
 * field pointer or a parameter changes.  The clock state (step index, sub_t, frame index) lives in
 * the workspace: it starts at step -1 and is set by pfm_step_reset; pfm_step_info reads it and the
 * two solves' statistics (a synchronization point).  poisson.max_iters must be >= 0 (the loop
 * ends on the device); p_mid may be NULL (the midpoint solve then starts from zero). */
typedef struct pfm_step_params {
  double CFL;                 /* hyperparameters.CFL */
  double visualize_dt;        /* hyperparameters.visualize_dt */
  int save_frame_each_step;   /* hyperparameters.save_frame_each_step */
  int reinit_every;           /* hyperparameters.reinit_every */
  int reinit_every_grad_m;    /* hyperparameters.reinit_every_grad_m */
  int use_midpoint_vel;       /* hyperparameters.use_midpoint_vel */
  int reinit_particle_pos;    /* hyperparameters.reinit_particle_pos */
  pfm_solve_opts poisson;     /* both projections */
} pfm_step_params;

typedef struct pfm3_step_fields {
  float* u[3];      /* face velocity, in/out */
  float* u_mid[3];  /* midpoint velocity (scratch) */
  float* w[3];      /* P2G weights (scratch) */
  float* p;         /* pressure of the final projection (warm start in, result out) */
  float* p_mid;     /* pressure of the midpoint projection, or NULL */
  const float* seeds;  /* [3][P] reseeding positions */
  float* pos;       /* [3][P] */
  float* init_imp;  /* [3][P] */
  float* T_init;    /* [3][3][P] */
  float* T_gm;      /* [3][3][P] */
  float* init_C;    /* [3][3][P] */
} pfm3_step_fields;

typedef struct pfm2_step_fields {
  float* u[2];
  float* u_mid[2];
  float* w[2];
  float* psi_grid[2];  /* P2G of the reference map psi ([F][2] per family), or NULL */
  float* p;
  float* p_mid;
  const float* seeds;  /* [2][P] */
  float* pos;       /* [2][P] */
  float* imp;       /* [2][P] */
  float* init_imp;  /* [2][P] */
  float* psi;       /* [2][P] */
  float* T;         /* [2][2][P] */
  float* T_init;    /* [2][2][P] */
  float* T_gm;      /* [2][2][P] */
  float* init_C;    /* [2][2][P] */
  float* C;         /* [2][2][P] */
} pfm2_step_fields;

typedef struct pfm_step_info_t {
  int step;           /* index i of the last step */
  int ik;             /* step of the last reseed (the gradient schedule's origin) */
  int frame_idx;
  int output_frame;   /* the last step ended a frame */
  int reinit;         /* the last step reinitialised the flow map (j == 0) */
  int reseed;         /* ... and reseeded the particles */
  int gradm_reinit;   /* the last step reinitialised the flow-map gradient (k == 0) */
  double dt;          /* its dt */
  double sub_t;
  float max_speed;
  int iterations[2];  /* MGPCG iterations: midpoint [0], final [1] */
  int converged[2];
  double rTr[2];
  int history[64][2]; /* iterations of the two solves of step s at s % 64 (the last 64 steps) */
} pfm_step_info_t;

int pfm3_step(pfm_handle* h, const pfm3_step_fields* f, const pfm_step_params* p, void* stream);
int pfm2_step(pfm_handle* h, const pfm2_step_fields* f, const pfm_step_params* p, void* stream);
/* Sets the step clock: the next step is i + 1; ik, sub_t and frame_idx as the reference's loop
 * variables (restart from a checkpoint).  pfm_step_reset(h, -1, 0, 0, 0) is a fresh start. */
int pfm_step_reset(pfm_handle* h, int i, int ik, double sub_t, int frame_idx, void* stream);
/* Forgets the previous solutions kept for warm_start 2 and 3 (a new simulation on the same handle and
 * pressure buffers); asynchronous on `stream`.  No counterpart in the reference, whose solves
 * start from zero (3D/mgpcg.py:63-79). */
int pfm_reset_warm_history(pfm_handle* h, void* stream);
/* SYNCHRONIZATION POINT: the state after the last step.  Also adds the kernels the step graphs
 * ran to pfm_launch_count. */
int pfm_step_info(pfm_handle* h, pfm_step_info_t* info, void* stream);

/* ---- batches of independent scenes -------------------------------------------------------------
 * A batch advances many scenes (of any sizes, 2D and 3D mixed) one step with ONE graph launch: the
 * graph holds every scene's whole step (as pfm3_step / pfm2_step) as an independent branch, so the
 * GPU runs the scenes' kernels concurrently and the small scenes fill the SMs the large ones leave
 * idle.  Each scene keeps its own handle (whose workspace holds its step clock and solver state;
 * a handle can be in one batch once) and its own fields; results are bitwise those of stepping the
 * scenes one by one.  The graph is built on the first pfm_batch_step after the last add.  Errors
 * of batch calls are reported by pfm_batch_last_error; pfm_step_info / pfm_step_reset work on each
 * scene's handle. */
typedef struct pfm_batch pfm_batch;
int pfm_batch_create(pfm_batch** out);
int pfm_batch_destroy(pfm_batch* b);
int pfm_batch_add3(pfm_batch* b, pfm_handle* h, const pfm3_step_fields* f, const pfm_step_params* p);
int pfm_batch_add2(pfm_batch* b, pfm_handle* h, const pfm2_step_fields* f, const pfm_step_params* p);
int pfm_batch_step(pfm_batch* b, void* stream);
const char* pfm_batch_last_error(const pfm_batch* b);
/* Work-list form of the batch (on = 1; 0 = the branch form above, the default): each scene's step
 * runs in its own branch up to the setup of an MGPCG solve (3D/mgpcg.py:202-280 inside the step
 * loop of 3D/run_3D.py:716-822, 2D/run_2D.py:772-909); then one WHILE node advances every scene's
 * solver iterations with persistent kernels over a work list of (scene, thread block) items, one
 * launch per kernel of the iteration for the whole batch, a converged scene skipping its items;
 * the branches continue behind it.  Same results bit for bit.  The scenes must share the dimension,
 * the midpoint flag and the solver options, and leave PFM_TUNE_SMOOTH_TMA at 0 (else
 * pfm_batch_step returns PFM_ERR_ARG); at most 128 scenes.  Takes effect at the next step. */
int pfm_batch_set_worklist(pfm_batch* b, int on);

/* ---- the reference's alternative ("evolve m") dataflow ---------------------------------------
 * Kernels the reference defines beside its live step (their call sites in 3D/run_3D.py:795-808
 * are commented out).  grad_T_init is the three per-particle 3x3 matrices grad_T_init_x/y/z as
 * [3 (row vector r)][3][3][P]. */

/* RK4_T_and_T_grad_m_forward (3D/run_3D.py:221-292): RK4 of pos [3][P] and of two Jacobian sets
 * T and T_grad_m ([3][3][P] each, must not alias) with the same velocity gradient; in place. */
int pfm3_rk4_T_and_T_grad_m_forward(pfm_handle* h, float* pos, float* T, float* T_grad_m, const float* u_x,
                                    const float* u_y, const float* u_z, float dt, void* stream);
/* update_particles_imp (3D/run_3D.py:395-401): imp = cols(T) @ init_imp. */
int pfm3_update_imp(pfm_handle* h, float* imp, const float* init_imp, const float* T, void* stream);
/* update_particles_grad_m (3D/run_3D.py:412-428): C_r = grad_T_init_r @ init_imp + (T^T init_C T)_r
 * with T = rows(T) ([3][3][P]); grad_T_init may be NULL (zero). */
int pfm3_update_grad_m(pfm_handle* h, float* C, const float* init_C, const float* T, const float* grad_T_init,
                       const float* init_imp, void* stream);
/* compute_dT_dx (3D/run_3D.py:353-390): grad_T_init of every particle from the particles in the
 * 4x4x4 cells around its initial position init_pos, using the cell lists of the current positions
 * pos (get_particles_id_in_every_cell, at most cap particles per cell in particle-index order) and
 * the neighbours' T ([3][3][P]).  Distances are in world units, as the reference writes them.
 * Neighbour cells outside the grid are skipped (the reference reads outside its fields there). */
int pfm3_compute_dT_dx(pfm_handle* h, const float* pos, const float* init_pos, const float* T, int cap,
                       float* grad_T_init, void* stream);

/* ---- scalar (smoke) transport ---------------------------------------------------------------
 * The smoke grid is cell-centred AoS like the reference's ti.Vector.field(4, float, shape=res):
 * smoke [nx][ny][nz][4] f32 (3D, 16-byte aligned), [nx][ny][3] (2D).  Particle smoke is SoA:
 * smoke_p [4][P]; the per-particle 3x4 smoke gradient is [3][4][P] (row r = d/dx_r, column = channel).
 * psi_x/psi_y/psi_z are the backward-map face grids [F][3] (3D) / [F][2] (2D) that pfm3_midpoint /
 * pfm2_midpoint write through psi_out. */

/* init_particles_smoke (3D/init_conditions.py:275-279) via interp_u_MAC_smoke / interp_grad_2_smoke
 * (3D/taichi_utils.py:379-428): smoke value and gradient at the particle positions pos [3][P].
 * smoke_p and grad_smoke may be NULL. */
int pfm3_init_particles_smoke(pfm_handle* h, const float* pos, const float* smoke, float* smoke_p,
                              float* grad_smoke, void* stream);

/* P2G_smoke (3D/run_3D.py:554-593): APIC transfer of the particle smoke with the affine term
 * dpos . ((cols(T_gm) @ cols(T_init)) @ init_grad_smoke) when use_apic_smoke is nonzero
 * (hyperparameters.use_APIC_smoke), normalised by the weight sums (weight [nx][ny][nz]) and clamped
 * to [0, 1] where the weight is positive.  Deterministic (bin sort + cell tiles, no float atomics).
 * Overwrites the P2G records of pfm3_rk4_p2g_records in the workspace. */
int pfm3_p2g_smoke(pfm_handle* h, const float* smoke_p, const float* init_grad_smoke, const float* pos,
                   const float* T_gm, const float* T_init, int use_apic_smoke, float* smoke, float* weight,
                   void* stream);

/* advect_smoke (3D/run_3D.py:315-323): smoke1 = trilinear interp_1 of smoke0 at the cell-centre
 * average of the six face backward maps; clamp_smoke (3D/run_3D.py:326-334): clamps smoke1 to the
 * min/max of the eight smoke0 corners there.  dx is the reference's kernel argument. */
int pfm3_advect_smoke(pfm_handle* h, const float* smoke0, float* smoke1, const float* psi_x,
                      const float* psi_y, const float* psi_z, float dx, void* stream);
int pfm3_clamp_smoke(pfm_handle* h, const float* smoke0, float* smoke1, const float* psi_x,
                     const float* psi_y, const float* psi_z, float dx, void* stream);
/* advect_smoke (2D/run_2D.py:444-450), 3-channel smoke. */
int pfm2_advect_smoke(pfm_handle* h, const float* smoke0, float* smoke1, const float* psi_x,
                      const float* psi_y, float dx, void* stream);

/* ---- diagnostics ------------------------------------------------------------------------------ */

/* add_fields (3D/taichi_utils.py:18-21, 2D/taichi_utils.py:13-16): dest = f1 + multiplier * f2,
 * and scale_field (3D/taichi_utils.py:13-16, 2D/taichi_utils.py:8-11): result = alpha * a, over n
 * floats of any field shape (f32, the product rounded before the sum).  No handle. */
int pfm_add_fields(const float* f1, const float* f2, float multiplier, float* dest, int64_t n, void* stream);
int pfm_scale_field(const float* a, float alpha, float* result, int64_t n, void* stream);
/* get_central_vector (3D/taichi_utils.py:80-85): vc [nx][ny][nz][3] = face averages. */
int pfm3_get_central_vector(pfm_handle* h, const float* u_x, const float* u_y, const float* u_z, float* vc,
                            void* stream);
/* curl (3D/taichi_utils.py:56-78): w [nx][ny][nz][3], central differences of vc with clamped
 * neighbours and 1/(2 dx). */
int pfm3_curl(pfm_handle* h, const float* vc, float* w, float dx, void* stream);
/* get_central_vector (2D/taichi_utils.py:50-55): vc [nx][ny][2]. */
int pfm2_get_central_vector(pfm_handle* h, const float* u_x, const float* u_y, float* vc, void* stream);
/* curl (2D/taichi_utils.py:96-104): scalar vorticity w [nx][ny]. */
int pfm2_curl(pfm_handle* h, const float* vc, float* w, float dx, void* stream);

/* ---- initial conditions --------------------------------------------------------------------- */

/* add_vortex_ring_and_smoke (3D/init_conditions.py:29-56): adds the ring's velocity to vc (as
 * pfm3_add_vortex_ring) and its marker sum(curve_length * exp(-(r/delta)^3)) to smoke[..][3], then
 * sets every cell whose marker exceeds 0.002 to (color, 1) and every other cell to 0.
 * smoke [nx][ny][nz][4], 16-byte aligned; c/unit_x/unit_y/color are host arrays. */
int pfm3_add_vortex_ring_and_smoke(pfm_handle* h, float w, float rad, float delta, const float c[3],
                                   const float unit_x[3], const float unit_y[3], const float color[3],
                                   int num_samples, float* vc, float* smoke, void* stream);

/* add_vortex_ring (3D/init_conditions.py:10-22): adds the Biot-Savart velocity of a ring of
 * strength w, radius rad and core delta (mollifier 1-exp(-(r/delta)^3)) centred at c in the plane
 * spanned by unit_x/unit_y, sampled with num_samples points, to the cell-centred vector field
 * vc [nx][ny][nz][3] (cell centres at (I + 0.5) dx).  c/unit_x/unit_y are host arrays. */
int pfm3_add_vortex_ring(pfm_handle* h, float w, float rad, float delta, const float c[3],
                         const float unit_x[3], const float unit_y[3], int num_samples, float* vc,
                         void* stream);
/* split_central_vector (3D/taichi_utils.py:87-100, 2D/taichi_utils.py:56-67): face velocity =
 * average of the two adjacent cell-centred values (clamped at the walls).  vc [cells][dim]. */
int pfm_split_central_vector(pfm_handle* h, const float* vc, float* u_x, float* u_y, float* u_z,
                             void* stream);

/* Jittered particle seeding (particles uniformly jittered from a seed): each cell
 * holds ppc_axis^dim particles, one per sub-cell, at (sub-lattice index + U) * dx / ppc_axis with
 * U from a counter-based splitmix64 hash of (seed, particle index, axis).  Order: the lines of
 * cells along the last axis in turn, each in groups of 16 cells; inside a group
 * [leading sub-indices][cell][last sub-index] (8 particles per cell: 32 consecutive particles
 * are 16 neighbouring cells with the same leading sub-cell, which keeps a warp's interpolation
 * stencils on shared rows).  P must equal ppc_axis^dim * cells.  pos [dim][P].  Bit-identical to
 * pfm.sim.jittered() on the host. */
int pfm_seed_jittered(pfm_handle* h, uint64_t seed, int ppc_axis, float* pos, void* stream);

/* ---- the MGPCG solver alone ----------------------------------------------------------------- */

/* MGPCG.init(r, k) + solve() + get_result(x) (3D/mgpcg.py:71-90, 202-280): solves the scaled
 * Poisson problem lap(x) = k r for a caller-given cell field r [cells] (Poisson() uses the
 * divergence with k = -1, 3D/mgpcg.py:420-423).  x_out [cells] receives the solution.
 * SYNCHRONIZATION POINT. */
int pfm_mgpcg_solve(pfm_handle* h, const float* r, float k, float* x_out, const pfm_solve_opts* opts,
                    pfm_solve_stats* stats, void* stream);

/* The pieces of MGPCG_3/MGPCG_2.Poisson (3D/mgpcg.py:359-418, 2D/mgpcg.py:293-335); u_z is NULL
 * in 2D.  apply_bc zeroes the normal velocity on Neumann walls; divergence writes
 * div_out [cells] = sum of face differences (unit spacing); subtract_grad_p subtracts the
 * pressure difference p [cells] from every face (zero pressure outside the grid), without the
 * wall reset (Poisson calls apply_bc after it). */
int pfm_apply_bc(pfm_handle* h, float* u_x, float* u_y, float* u_z, void* stream);
int pfm_divergence(pfm_handle* h, const float* u_x, const float* u_y, const float* u_z, float* div_out,
                   void* stream);
int pfm_subtract_grad_p(pfm_handle* h, float* u_x, float* u_y, float* u_z, const float* p, void* stream);

/* The Boussinesq smoke plume that trains and evaluates the learned warm start (the reference has
 * no forces or plume; these run around its unchanged step).  rho is a cell field [nx][ny][nz].
 *  - plume_source: rho = value in the cells whose centre lies within `radius` of (cx, cy, cz);
 *  - advect_density: rho1(x) = rho0(x - dt u(x)), u averaged from the faces to the cell centre,
 *    trilinear sampling clamped to the cell centres (rho0 != rho1);
 *  - add_buoyancy_impulse: the force coef * rho(x_p) along `axis` applied to each particle's
 *    impulse: init_imp += M^-1 f with M = cols(T_gm) cols(T_init), the map P2G applies to init_imp
 *    (3D/run_3D.py:462-475), so the impulse P2G sees grows by f (coef = dt * buoyancy). */
int pfm3_plume_source(pfm_handle* h, float* rho, float cx, float cy, float cz, float radius, float value,
                      void* stream);
int pfm3_advect_density(pfm_handle* h, const float* rho0, float* rho1, const float* u_x, const float* u_y,
                        const float* u_z, float dt, void* stream);
int pfm3_add_buoyancy_impulse(pfm_handle* h, const float* pos, const float* T_gm, const float* T_init, float* init_imp,
                              const float* rho, float coef, int axis, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Learned warm start: the layers of the pressure U-Net (the learned variant beside the solver;
 * the reference has no network -- these entry points serve pfm.nn, which predicts an initial
 * pressure that MGPCG (3D/mgpcg.py:202-280) then refines to the same residual).
 *
 * Activations are BF16 "channel-blocked": C channels on an d0 x d1 x d2 grid (d2 fastest) are
 * [C/8][d0][d1][d2][8].  Weights are f32 masters W [cout][cin][27] (tap = 9 a + 3 b + c for the
 * offsets (a-1, b-1, c-1) along d0, d1, d2: cross-correlation with zero padding), packed to BF16
 * by pfm_nn_pack_weights.  Every convolution accumulates in F32 on the tensor cores.  `err` is a
 * device int that a kernel sets nonzero if one of its bounded waits gave up (a CUDA fault
 * otherwise never passes silently: the caller checks it after synchronizing).
 * ------------------------------------------------------------------------------------------- */
typedef struct pfm_conv3_args {
  int d0, d1, d2;       /* grid */
  const void* x1;       /* input, c1 channels (multiple of 16) */
  int c1;
  const void* x2;       /* optional second input concatenated after x1 (c2 multiple of 16, or 0) */
  int c2;
  const void* w;        /* packed [27][(c1+c2)/8][npad][8], npad = cout rounded up to 16 */
  const float* bias;    /* [cout] or NULL */
  int cout;             /* output channels, <= 128 */
  int relu;             /* 1: max(0, .) */
  void* y1;             /* BF16 channel-blocked output of channels [0, cy1) */
  int cy1;
  void* y2;             /* channels [cy1, cout) (NULL if cy1 == cout) */
  float* yf;            /* if not NULL: F32 planar output [cout][d0][d1][d2] instead of y1/y2 */
  const float* yf_scale;/* device scalar multiplying yf (NULL: 1) */
  int* err;
} pfm_conv3_args;

typedef struct pfm_conv3_wgrad_args {
  int d0, d1, d2;
  const void* x1;       /* the layer's input(s), as in pfm_conv3_args */
  int c1;
  const void* x2;
  int c2;
  const void* dy;       /* gradient of the layer's pre-activation output, cdy channels (multiple of 8) */
  int cdy;
  int cout;             /* real output channels (<= cdy) */
  float* dw;            /* out: dL/dW [cout][c1+c2][27], overwritten */
  float* partial;       /* device workspace of pfm_nn_wgrad_workspace bytes */
  size_t partial_bytes;
  int* err;
} pfm_conv3_wgrad_args;

/* 3x3x3 convolution, stride 1, zero padding (forward, or the data gradient with flipped weights). */
int pfm_nn_conv3(const pfm_conv3_args* a, void* stream);
/* Weight gradient dW = sum over voxels of x(v + tap) dy(v); deterministic. */
int pfm_nn_conv3_wgrad(const pfm_conv3_wgrad_args* a, void* stream);
int pfm_nn_wgrad_workspace(const pfm_conv3_wgrad_args* a, size_t* bytes);
/* Packs W [cout][cin][27] into [27][kin/8][npad][8] BF16 for the forward (flip 0: rows = cout,
 * K = cin) or the data gradient (flip 1: rows = cin, K = cout, taps mirrored). */
int pfm_nn_pack_weights(const float* W, int cout, int cin, int flip, int kin, int npad, void* wp, void* stream);
/* A scalar field f [d0][d1][d2] -> 16-channel block tensor, channel 0 = f * (*inv_scale). */
int pfm_nn_pack_scalar(const float* f, int d0, int d1, int d2, const float* inv_scale, void* x, void* stream);
/* mode 0: 2x2x2 average pool of the fine grid d0 x d1 x d2; 1: its backward; 2: nearest
 * upsampling to the fine grid; 3: its backward (sum of the 8 children). */
int pfm_nn_resample(const void* in, void* out, int channels, int d0, int d1, int d2, int mode, void* stream);
/* mode 0: g *= (y > 0) (ReLU backward); mode 1: g += y.  `elements` = channels x voxels. */
int pfm_nn_elementwise(void* g, const void* y, size_t elements, int mode, void* stream);
/* floats of scratch that pfm_nn_bias_grad / pfm_nn_loss need for `channels` channels */
size_t pfm_nn_scratch_floats(int channels);
/* db[c] = sum over voxels of dy channel c, c < cout (deterministic). */
int pfm_nn_bias_grad(const void* dy, int channels, int d0, int d1, int d2, int cout, float* db, float* scratch,
                     void* stream);
/* e = pred - target * (*inv_scale): out4 = {mean(e^2) - mean(e)^2, mean e, 1 / rms(e), rms(e)};
 * with grad != NULL also dL/dpred as channel 0 of a 16-channel block tensor.  pred = NULL gives
 * the RMS of the target (the scale of a right-hand side). */
int pfm_nn_loss(const float* pred, const float* target, const float* inv_scale, int d0, int d1, int d2,
                float* out4, void* grad, float* scratch, void* stream);
/* Adam step (bias-corrected, step >= 1) on f32 parameters with the gradient times gscale. */
int pfm_nn_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2,
                float eps, int step, float gscale, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PFM_H_ */
