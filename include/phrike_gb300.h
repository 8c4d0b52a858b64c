/*
 * phrike_gb300 — C ABI of the GB300 pseudo-spectral Euler step engine.
 *
 * Every entry point takes plain pointers (device pointers for field data),
 * sizes and a CUDA stream handle passed as void* (a cudaStream_t; NULL is the
 * legacy default stream), and returns an int status (PS_OK = 0).  On failure
 * ps_last_error() returns a thread-local message.  Field arrays are float32,
 * component-first and C-contiguous: (ncomp, [Nz,] [Ny,] Nx), x fastest — the
 * layout of the reference's state arrays (phrike/grid.py:779-780, 1361).
 *
 * Each declaration names the reference interface it replaces (paths inside
 * the reference project, file:line).  A Python binding over ctypes lives in
 * phrike_gb300/_lib.py.
 */
#ifndef PHRIKE_GB300_H
#define PHRIKE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define PS_OK 0
#define PS_ERR_INVALID 1     /* bad argument, null pointer, inconsistent descriptor */
#define PS_ERR_UNSUPPORTED 2 /* grid size / basis / equation set not supported     */
#define PS_ERR_CUDA 3        /* CUDA runtime error                                  */
#define PS_ERR_OOM 4         /* device allocation failed                            */

/* basis per axis */
#define PS_BASIS_FOURIER 0
#define PS_BASIS_LEGENDRE 1

/* equation sets */
#define PS_EQ_EULER 0
#define PS_EQ_MHD 1 /* 1D, 2D (2.5D) and 3D ideal/resistive MHD, 8 components
                       [rho, rho u (3), E, B (3)], periodic Fourier grids
                       (equations.py:659-1100, SpectralSolverMHD,
                       solver.py:840-1049, 1165-1174); 3D: 8..256 points per axis */

/* arithmetic of the LGL differentiation-matrix contractions */
#define PS_GEMM_FP32 0   /* float32 operands, float32 accumulate                 */
#define PS_GEMM_FP64 1   /* float64 operands and accumulate (flux in float64)     */
#define PS_GEMM_BF16X3 2 /* split bf16: hi*hi + hi*lo + lo*hi, float32 accumulate,
                            on tcgen05 tensor cores                              */
#define PS_GEMM_BF16X3_SIMT 3 /* the same split arithmetic on CUDA cores (for checks) */

typedef struct ps_plan_s* ps_plan;

/*
 * One solve: grid, basis, equations and step options.
 * Mirrors the constructor arguments of Grid1D/2D/3D (grid.py:170-181,
 * 782-797, 1364-1376), EulerEquations1D/2D/3D(gamma) (equations.py:217,
 * 322, 551) and SpectralSolver1D/2D/3D (solver.py:156, 565, 1262).
 */
typedef struct {
  int ndim;              /* 1, 2 or 3                                         */
  int n[3];              /* points along x, y, z (unused axes: 1)             */
  double length[3];      /* Lx, Ly, Lz                                        */
  int basis[3];          /* PS_BASIS_*                                        */
  int equations;         /* PS_EQ_*                                           */
  double gamma;          /* adiabatic index                                   */
  int dealias;           /* 2/3-rule mask (grid.py:47-54)                     */
  int filter_enabled;    /* exponential filter (grid.py:57-63)                */
  int filter_p;          /* filter order p                                    */
  double filter_alpha;   /* filter strength alpha                             */
  int filter_interval;   /* cadence of the end-of-step filter (1D/2D)         */
  double gravity[3];     /* constant gravity (solver.py:82-91); 0 = off       */
  double cfl;            /* CFL number for ps_compute_dt                      */
  int gemm_precision;    /* PS_GEMM_* (LGL grids; ignored for Fourier)        */
  /* PS_EQ_MHD options (grid.mhd_config of the reference, solver.py:871-880) */
  double mhd_rho_min;          /* clamp floors (default 1e-10, 1e-12)          */
  double mhd_p_min;
  int mhd_project_substages;   /* project B after every RK stage (default 1)   */
  int mhd_divergence_clean;    /* 1: Helmholtz projection, 0: none (default 1) */
  double mhd_resistivity;      /* eta: rhs_B += eta lap(B) (solver.py:945-950)  */
  double mhd_viscosity;        /* nu: rhs_(rho u) += nu lap(rho u) (951-954)    */
  /* Artificial viscosity, 1D/2D Euler (SpectralArtificialViscosity,
   * artificial_viscosity.py:37-403): rhs_c += div(w_c nu grad U_c) with
   * nu = av_nu_max ((s > av_s_min ? s : 0) / av_s_ref)^av_p and
   * s = clip(|grad q| / (|q| + av_epsilon) / av_s_ref, 0, 1), or nu constant. */
  int av_mode;                 /* PS_AV_OFF, PS_AV_SENSOR, PS_AV_CONSTANT       */
  int av_sensor;               /* PS_AV_Q_*: the sensor variable q              */
  double av_nu_max, av_nu_constant, av_s_ref, av_s_min, av_p, av_epsilon;
  double av_weight[5];         /* w_c per state component                       */
  /* Fixed-step scheme of ps_step_rk4 / ps_run_steps / ps_run_cfl: classical
   * RK4 (default) or the midpoint RK2 of _rk2_step / _rk2_step_2d /
   * _rk2_step_3d / _rk_substages (solver.py:96-105, 492-500, 1211-1216,
   * 992-996), with the same clamp, projection and filter placement. */
  int scheme;                  /* PS_SCHEME_RK4 or PS_SCHEME_RK2                */
  /* Parabolic CFL factor of explicit MHD diffusion (mhd_config "cfl_diff",
   * solver.py:878-880): dt <= mhd_cfl_diff / (max(eta, nu) k^2_max).
   * Default 1. */
  double mhd_cfl_diff;
  /* 1D Legendre grids: boundary codes per side (left, right) and variable
   * (density, momentum, energy), index side * 3 + variable: 0 copy the
   * neighbouring interior value (Neumann), 1 set to zero (the momentum of a
   * wall), 2 leave unchanged (Grid1D.apply_boundary_conditions,
   * grid.py:620-735).  Default: walls, {0, 1, 0, 0, 1, 0}. */
  int lgl_bc1d[6];
  /* 2D Fourier plans: columns per tile of the strided passes, 4, 8 or 16 (at
   * most the plan's cap: 16 below 256-point y pencils, then 8 (Euler to 1023
   * points, MHD beyond), 4 for Euler from 1024); 0 (default): the plan's
   * heuristic.  The arithmetic of a pencil does not depend on it;
   * phrike_gb300/autotune.py picks it by timing. */
  int tile_cols;
  /* LGL x LGL plans with PS_GEMM_BF16X3: N tile of the tcgen05 contractions,
   * 64, 128, 176 or 256 columns; 0 (default): the smallest tile whose grid
   * fits one wave, else 256.  Every output element is the same dot product
   * for every tile; phrike_gb300/autotune.py picks it by timing. */
  int umma_n_tile;
} ps_plan_desc;

#define PS_SCHEME_RK4 0
#define PS_SCHEME_RK2 1

#define PS_AV_OFF 0
#define PS_AV_SENSOR 1
#define PS_AV_CONSTANT 2
#define PS_AV_Q_DENSITY 0
#define PS_AV_Q_PRESSURE 1 /* 1D: p; 2D: u_y, as the reference's sensor unpacks it */
#define PS_AV_Q_SPEED 2    /* |u| (1D only)                                     */

/* Fill a descriptor with the reference defaults for `ndim` (dealias on,
 * filter off with p=8, alpha=36, interval 1, gamma 1.4, cfl 0.4/0.3/0.25,
 * float32 LGL contractions). */
int ps_plan_desc_init(ps_plan_desc* desc, int ndim);

/* Device scratch a plan allocates at creation (bytes), for HBM admission. */
int ps_plan_scratch_bytes(const ps_plan_desc* desc, size_t* bytes);
int ps_batch_scratch_bytes(const ps_plan_desc* desc, int nsolve, size_t* bytes);

/* Build spectral tables and allocate scratch on the current device.
 * Replaces Grid*.__post_init__ + _setup_fourier_backend (grid.py:183-383,
 * 806-992, 1378-1495) and solver construction (solver.py:156-232).
 * A 2D descriptor with PS_BASIS_LEGENDRE on both axes makes an LGL x LGL
 * plan (Grid2D with basis_x = basis_y = "legendre", grid.py:806-840, and
 * LegendreLobattoBasis2D, basis/legendre.py:894-934): n >= 3 nodes per axis,
 * solid walls (bc "dirichlet", grid.py:994-1154) applied in place to every
 * stage input and after every step, the 2D positivity clamp after every RK
 * stage, the nodal filter (legendre.py:825-859) when enabled.
 * Fourier axis lengths: any N whose prime factors are 2, 3 and 5, from 2 to
 * 4096 (the reference's grids take any N, grid.py:47-63, 87-115).  Powers of
 * two from 8 to 1024 (to 4096 in 1D) run on register-resident pencils; other
 * lengths run on mixed-radix passes with the same results, for the Euler
 * equations without artificial viscosity (MHD and viscosity return
 * PS_ERR_UNSUPPORTED there, and so does 1D adaptive stepping). */
int ps_plan_create(const ps_plan_desc* desc, ps_plan* out);
int ps_plan_destroy(ps_plan plan);

/* A batch: nsolve independent solves of the same grid in one plan.  Every
 * field argument of the calls below then holds all solves back to back,
 * [nsolve][ncomp][cells], and per-solve outputs are arrays of nsolve entries.
 * A plain plan is a batch of one.  Replaces a Python loop over independent
 * SpectralSolver*.run calls (solver.py:338-422 per solve). */
int ps_batch_create(const ps_plan_desc* desc, int nsolve, ps_plan* out);
int ps_plan_nsolve(ps_plan plan);
/* Steps taken by each solve in ps_run_cfl calls so far (host array of
 * nsolve ints, read synchronously). */
int ps_plan_steps_done(ps_plan plan, int* host_steps);

/* rhs = -(sum_a d/dx_a F_a(U)) for U (ncomp fields).  Replaces
 * _compute_rhs / _compute_rhs_2d / _compute_rhs_3d (solver.py:62-93,
 * 428-466, 1177-1208). */
int ps_rhs(ps_plan plan, const float* U, float* rhs, void* stream);

/* One fixed-dt RK4 step in place, including the positivity clamp (1D/2D)
 * and the end-of-step filter with the reference cadence.  Replaces
 * SpectralSolver*.step / _fixed_step (solver.py:242-269, 623-648,
 * 1313-1337).  If d_dt is non-NULL the step sizes are read from device memory
 * (one double per solve) and `dt` is ignored, so the call can be captured in
 * a graph. */
int ps_step_rk4(ps_plan plan, float* U, double dt, const double* d_dt, void* stream);

/* nsteps fixed-dt RK4 steps in place (same semantics as nsteps calls of
 * ps_step_rk4; consecutive steps share fused filter passes). */
int ps_run_steps(ps_plan plan, float* U, int nsteps, double dt, const double* d_dt, void* stream);

/* Up to nsteps CFL-driven RK4 steps with the time loop on the device: per
 * solve, dt = min(cfl * h_min / max wave speed, t_end - t) from the state at
 * the start of each step, t advances in d_t (nsolve doubles, updated in
 * place), and a solve stops once t >= t_end - 1e-12.  No host
 * synchronisation, so the call can be captured in a CUDA graph.  For 2D/3D
 * grids the step loop is issued from the host, so nsteps is also the number
 * of steps launched (finished solves skip their work but the launches still
 * happen): advance in chunks and read d_t between chunks.  Replaces the
 * while-loop of SpectralSolver*.run (solver.py:384-417, 773-800, 1480-1505). */
int ps_run_cfl(ps_plan plan, float* U, int nsteps, double* d_t, const double* d_tend, void* stream);

/* Adaptive embedded Runge-Kutta (adaptive.py:23-437).  Methods: */
#define PS_ARK_RK23 0 /* Bogacki-Shampine 3(2)                                   */
#define PS_ARK_RK45 1 /* Dormand-Prince 5(4)                                     */
#define PS_ARK_RK78 2 /* the reference's simplified 8-stage "rk78" table        */
typedef struct ps_adaptive_desc {
  int method;            /* PS_ARK_*                                          */
  double rtol, atol;     /* tol = atol + rtol * max|U|                        */
  double safety_factor;  /* dt_new = dt * clip(safety (tol/err)^(1/order),    */
  double min_dt_factor;  /*                     min_dt_factor, max_dt_factor) */
  double max_dt_factor;
  int max_rejections;    /* forced acceptance after this many in a row        */
} ps_adaptive_desc;
/* The reference's defaults: rk45, rtol 1e-6, atol 1e-8, safety 0.9, factors
 * 0.1 and 5, 10 rejections (solver.py:182-193, adaptive.py:38-43). */
void ps_adaptive_desc_init(ps_adaptive_desc* ad);

/* Up to nattempts adaptive attempts per solve with every decision on the
 * device.  Replaces the adaptive branch of SpectralSolver*.run
 * (_adaptive_run_step, solver.py:295-323, 671-691, 1067-1084, 1360-1380).
 * Per solve, an attempt runs while t < t_end - 1e-12 (and, if d_tout is
 * non-NULL, while t + 1e-12 < t_out, so the host can record outputs at the
 * reference's times): dt = min(d_dt, t_end - t); the embedded pair gives
 * U_high and err = max|U_high - U_low|; the controller accepts when
 * err <= atol + rtol * max|U| (or after max_rejections rejections in a row)
 * and writes dt_next to d_dt.  An accepted attempt advances d_t and applies
 * the solver's post-step operator: the spectral filter (Euler), or filter,
 * clamp and projection (2D MHD).  The stage right-hand sides carry gravity;
 * 1D ones also carry artificial viscosity (the 2D/3D reference passes none
 * there).  No clamp inside the stages.
 * d_t, d_dt: nsolve doubles (in/out); d_tend: nsolve doubles; d_tout:
 * nullable; d_counts: nullable, nsolve x 2 ints to which accepted and
 * rejected attempts are added.  Consecutive-rejection counts stay in the plan
 * between calls (ps_adaptive_reset clears them).  The first call with a given
 * method allocates the stage storage (stages x state size): make it outside
 * any stream capture.  For 2D/3D grids nattempts is also the number of
 * attempt launch sequences issued (paused or finished solves skip their
 * work).  LGL grids return PS_ERR_UNSUPPORTED. */
int ps_run_adaptive(ps_plan plan, float* U, int nattempts, const ps_adaptive_desc* ad, double* d_t,
                    const double* d_tend, double* d_dt, const double* d_tout, int* d_counts, void* stream);
int ps_adaptive_reset(ps_plan plan, void* stream);

/* out = dx1/dy1/dz1(f) for nfields fields (axis 0 = x).  Replaces
 * Grid1D.dx1 (grid.py:512-522), Grid2D.dx1/dy1 (grid.py:1226-1252),
 * Grid3D.dx1/dy1/dz1 (grid.py:1705-1721). */
int ps_derivative(ps_plan plan, int axis, const float* f, float* out, int nfields, void* stream);

/* out = apply_spectral_filter(f) for nfields fields (may alias).  Replaces
 * Grid*.apply_spectral_filter (grid.py:524-538, 1254-1287, 1723-1726). */
int ps_filter(ps_plan plan, const float* f, float* out, int nfields, void* stream);

/* d_out (device floats, one per solve) = max wave speed of U with the reference's
 * per-dimension rule.  Replaces Euler*.max_wave_speed (equations.py:297-301,
 * 365-370, 609-620).  The result stays on the device. */
int ps_max_wave_speed(ps_plan plan, const float* U, float* d_out, void* stream);

/* d_out (device doubles, ncomp values per solve: mass, momenta..., energy) = plain
 * sums of the conserved quantities, accumulated in float64.  Replaces the
 * solvers' record() (solver.py:372-377, 741-767, 1439-1468).  For PS_EQ_MHD
 * the 8 values per solve are mass, momentum x/y/z, energy, magnetic energy,
 * cross helicity and 0 (MHDEquations2D.conserved_quantities,
 * equations.py:889-907). */
int ps_conserved(ps_plan plan, const float* U, double* d_out, void* stream);

/* LGL nodes, quadrature weights and differentiation matrix of one axis,
 * built on the device in float64: nodes ascending on [0, length], weights
 * of the reference interval [-1, 1], D[i][j] = d l_j / dx at x_i ([n][n],
 * row-major).  Replaces _legendre_gauss_lobatto_nodes_weights and
 * _stable_legendre_diff_matrix with the axis scaling of
 * LegendreLobattoBasis1D (basis/legendre.py:523-624, 694-729).  Any of the
 * three outputs may be NULL. */
int ps_lgl_build(int n, double length, double* d_nodes, double* d_weights, double* d_D, void* stream);

/* Apply the plan's boundary conditions to U in place: the solid walls of an
 * LGL x LGL plan (grid.py:1072-1154: left, right, top, bottom; density,
 * tangential momentum and energy copy the neighbouring line, the normal
 * momentum is zeroed).  A no-op for periodic Fourier plans, like
 * Grid*.apply_boundary_conditions there (grid.py:631-632, 1087-1089). */
int ps_apply_boundary_conditions(ps_plan plan, float* U, void* stream);

/* Helmholtz (Leray) projection of the in-plane field (Bx, By) in place,
 * div B = 0 to rounding: the Nyquist row and column are zeroed and
 * B_hat -= k (k . B_hat)/|k|^2.  Bx and By each hold nsolve fields of the
 * plan's 2D Fourier grid.  Replaces Grid2D.project_solenoidal
 * (grid.py:1297-1327). */
int ps_project_solenoidal(ps_plan plan, float* Bx, float* By, void* stream);

/* One-axis spectral operator on nf fields per solve (in place allowed):
 * PS_OP_P applies mask x filter along `axis` (0 = x), PS_OP_D the masked
 * derivative i k m s (Nyquist term dropped), PS_OP_L the masked second
 * derivative -k^2 m s (Nyquist kept).  Products of one-axis operators give
 * the grids' operators: dx1 = D_x P_y P_z, laplacian = L_x P_y P_z + P_x L_y P_z
 * + P_x P_y L_z (grid.py:569-579, 1329-1338, 1696-1703). */
#define PS_OP_P 0
#define PS_OP_D 1
#define PS_OP_L 2
int ps_axis_op(ps_plan plan, int axis, int op, const float* f, float* out, int nfields, void* stream);

/* The 3D projection of (Bx, By, Bz) in place for a 3D MHD plan: Nyquist
 * planes zeroed, B_hat -= k (k . B_hat)/|k|^2.  Replaces
 * Grid3D.project_solenoidal (grid.py:1649-1684). */
int ps_project_solenoidal_3d(ps_plan plan, float* Bx, float* By, float* Bz, void* stream);

/* The MHD state projection of SpectralSolverMHD._project_B
 * (solver.py:966-986) in place on U (PS_EQ_MHD plans): B projected, E
 * recomputed with the thermal pressure held fixed. */
int ps_project_state(ps_plan plan, float* U, void* stream);

/* Spectral interpolation of Fourier fields at arbitrary points:
 *   out[c][p] = Re( sum_k c_k F_k exp(i k . x_p) ) / N_total,  F = FFT(f_c),
 * c_k the plan's dealias mask x filter, k = 2 pi fftfreq(N)/L per axis, i.e.
 * the exact trigonometric interpolant the reference evaluates without finufft
 * (and to its eps = 1e-6 with it).  f holds nf (1..3) fields of the plan's
 * grid (solve 0), points is [ndim][npoints] float64 (x row, then y, z), out
 * [nf][npoints] float32.  Fourier plans only; see ps_tracer_method for the
 * interpolation (exact, O(npoints x cells), or NUFFT).
 * Replaces Grid1D.evaluate_fourier_at_points_1d (grid.py:581-618),
 * Grid2D.evaluate_fourier_at_points (grid.py:1180-1222) and the 3D single
 * and batched forms (grid.py:1520-1632). */
int ps_eval_points(ps_plan plan, const float* f, int nf, const double* points, int npoints, float* out,
                   void* stream);

/* How ps_eval_points and ps_tracers_step interpolate:
 *   PS_TRACERS_EXACT  the exact trigonometric interpolant, O(npoints x cells);
 *   PS_TRACERS_NUFFT  type-2 NUFFT interpolation (the method of the
 *                     reference's finufft branch, grid.py:611, 1214, 1555):
 *                     exponential-of-semicircle kernel, 8 points per axis on a
 *                     2x oversampled grid, within 1e-6 of the exact
 *                     interpolant; O(cells log cells + npoints); axes of
 *                     2^a 3^b 5^c points up to 2048;
 *   PS_TRACERS_AUTO   (default) NUFFT once npoints x cells exceeds 2^24 and the
 *                     grid allows it, else exact. */
#define PS_TRACERS_AUTO 0
#define PS_TRACERS_EXACT 1
#define PS_TRACERS_NUFFT 2
int ps_tracer_method(ps_plan plan, int method);

/* One leap-frog step of tracer particles in the velocity u_a = U[1+a]/U[0]
 * of the state U (solve 0), interpolated as in ps_eval_points:
 *   first != 0: prev = pos; pos += dt u        (Euler start)
 *   otherwise:  pos, prev = prev + 2 dt u, pos
 * then pos = pos mod L per axis (numpy's rule, result in [0, L)).  pos and
 * prev are [ndim][npoints] float64, updated in place; velocity_out
 * ([ndim][npoints] float32) receives the interpolated velocity when not
 * null.  Replaces FourierTracers1D/2D/3D.step (tracers.py:50-79, 103-148,
 * 178-236). */
int ps_tracers_step(ps_plan plan, const float* U, double* pos, double* prev, int npoints, int first, double dt,
                    float* velocity_out, void* stream);

/* Device status word of a plan, read synchronously: 0 = healthy; bit
 * PS_STATUS_TMA_TIMEOUT = a kernel gave up waiting for a tile load (bounded
 * wait) and its results are invalid.  No reference counterpart: the
 * reference raises Python exceptions only (grid.py:79-84, 305-308). */
#define PS_STATUS_TMA_TIMEOUT 1
int ps_plan_status(ps_plan plan, int* status);

/* Launch profiling: when enabled, every pass launch is bracketed by CUDA
 * events on its stream and tagged with its kind and the algorithmic bytes it
 * moves.  ps_profile_collect waits for the recorded events, fills per-kind
 * launch counts, elapsed milliseconds and bytes (arrays of nkinds entries,
 * indexed by PS_KIND_*) and clears the log.  No reference counterpart: the
 * reference has no built-in tracing (its timings are ad-hoc perf_counter
 * calls, benchmark_tracers.py:64-75). */
#define PS_KIND_X 0      /* x pass: flux + D_x / P_x               */
#define PS_KIND_Y 1      /* 3D y pass                              */
#define PS_KIND_LAST 2   /* last pass: rhs + RK4 stage (+ filter)  */
#define PS_KIND_OP 3     /* one-axis operator / filter pass        */
#define PS_KIND_STEP1D 4 /* 1D whole-step kernel                   */
#define PS_KIND_LGL_X 5  /* LGL: x flux + contraction with D_x     */
#define PS_KIND_LGL_Y 6  /* LGL: y flux + D_y contraction + stage  */
#define PS_NKINDS 7
int ps_profile_enable(ps_plan plan, int enable);
int ps_profile_collect(ps_plan plan, int nkinds, int* launches, double* ms, double* bytes);

/* Allocation-free right-hand side (no counterpart in the reference).
 * Same result as ps_rhs for a 2D or 3D Fourier Euler grid, but it takes the
 * descriptor by value instead of a plan and allocates no device memory: the
 * spectral tables and pass intermediates live in one static device array of
 * PS_RHS_STATIC_MAX_CELLS cells' worth of scratch (about 6.6 MB, held by every
 * GPU that loads the library until the process exits).  For callers that
 * cannot call cudaMalloc where they evaluate a right-hand side: code inside a
 * stream capture, frameworks that own all device memory through their own
 * pool, allocation-free real-time loops.  Grids of more cells return
 * PS_ERR_UNSUPPORTED.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress); make it before any stream capture.  Calls
 * share the array: calls that overlap on the GPU race, so keep them on one
 * stream. */
#define PS_RHS_STATIC_MAX_CELLS 65536
int ps_rhs_static(const ps_plan_desc* desc, const float* U, float* rhs, void* stream);

/* Columns per strided-pass tile the plan uses (2D Fourier plans; 0 otherwise). */
int ps_plan_tile_cols(ps_plan plan);

/* Number of state components (ndim + 2 for Euler). */
int ps_plan_ncomp(ps_plan plan);

/* Thread-local message of the last failed call ("" if none). */
const char* ps_last_error(void);

/* Library version string. */
const char* ps_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PHRIKE_GB300_H */
