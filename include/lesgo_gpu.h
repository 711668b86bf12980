/*
 * lesgo_gpu.h -- C ABI of the GB300-native LESGO time-step library.
 *
 * The library replaces the per-timestep hot path of LESGO (lesgo-jhu/lesgo):
 * the x-y spectral derivatives, the staggered z stencils, the Lagrangian
 * scale-dependent dynamic SGS model, the equilibrium wall model, the stress
 * divergence, the 3/2-dealiased convective term, the FFT + tridiagonal
 * pressure solve, the actuator-disk forcing and the AB2 advance / projection.
 * Every field lives in GPU memory; host arrays are only touched by the
 * explicit set/get/upload/download calls.
 *
 * Conventions shared with the reference:
 *  - 3-D arrays use the reference's Fortran layout (ld, ny, lbz:nzhi),
 *    column-major, FP64, ld = 2*(nx/2+1); the serial reference uses
 *    lbz = 1 (p: lbz = 0) and nz = Nz+1 (param.f90:49-55,
 *    input_util.f90:196-235).  Host <-> device copies are flat memcpys of
 *    whole (ld, ny) planes.
 *  - Every entry point returns an int status (LESGO_OK = 0) and never
 *    aborts; lesgo_gpu_last_error() describes the last failure.  The
 *    reference instead prints and stops (messages.f90:228-239,
 *    tridag_array.f90:190-193).
 *  - One host thread per handle; each handle owns one CUDA stream.
 */
#ifndef LESGO_GPU_H
#define LESGO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  LESGO_OK = 0,
  LESGO_ERR_ARG = 1,          /* bad argument or handle                    */
  LESGO_ERR_CUDA = 2,         /* CUDA runtime failure                      */
  LESGO_ERR_UNSUPPORTED = 3,  /* configuration outside the built model set */
  LESGO_ERR_NOMEM = 4,        /* device allocation refused                 */
  LESGO_ERR_NUMERIC = 5       /* zero pivot in the tridiagonal solve       */
};

/* ---- precision forms ---------------------------------------------------- */
enum {
  LESGO_FP64 = 0,   /* plain FP64 drop-in                                    */
  LESGO_MIXED = 1,  /* FP32 fields and transforms; FP64 pressure RHS,
                       tridiagonal solve, kx=ky=0 mode and wall log law      */
  LESGO_FP64_DW = 2 /* FP64 fields and pointwise arithmetic; the x-y
                       transforms in double-word (FP32 pair, 48-bit
                       significand) arithmetic on the FP32 pipe              */
};

/* ---- field identifiers (sim_param.f90:300-365, sgs_param.f90:30-184) ---- */
enum {
  LESGO_U = 0, LESGO_V, LESGO_W,
  LESGO_DUDX, LESGO_DUDY, LESGO_DUDZ,
  LESGO_DVDX, LESGO_DVDY, LESGO_DVDZ,
  LESGO_DWDX, LESGO_DWDY, LESGO_DWDZ,
  LESGO_RHSX, LESGO_RHSY, LESGO_RHSZ,
  LESGO_RHSX_F, LESGO_RHSY_F, LESGO_RHSZ_F,
  LESGO_TXX, LESGO_TXY, LESGO_TXZ, LESGO_TYY, LESGO_TYZ, LESGO_TZZ,
  LESGO_DIVTX, LESGO_DIVTY, LESGO_DIVTZ,
  LESGO_P, LESGO_DPDX, LESGO_DPDY, LESGO_DPDZ,
  LESGO_FXA, LESGO_FYA, LESGO_FZA,
  LESGO_S11, LESGO_S12, LESGO_S13, LESGO_S22, LESGO_S23, LESGO_S33,
  LESGO_NU_T, LESGO_CS_OPT2,
  LESGO_F_LM, LESGO_F_MM, LESGO_F_QN, LESGO_F_NN,
  LESGO_BETA, LESGO_TN_ALL, LESGO_EE_NOW,
  LESGO_NFIELDS
};

/* One actuator disk, lengths already divided by z_i (turbines.f90:759-785). */
typedef struct {
  double xloc, yloc, height, dia, thk;
  double theta1, theta2;   /* degrees */
  double Ct_prime;
} lesgo_turbine_t;

/* Run parameters: the subset of `param` (param.f90) and the TURBINES block
 * that the hot path reads, as lesgo.conf gives them.  Derived sizes
 * (nz, ld, lh, nx2, ny2, dx, dy, dz, tadv1/2, mean_p_force, delta) are
 * computed exactly as input_util.f90:196-235, 403-409, 534-542 and
 * sgs_param.f90:187. */
typedef struct {
  int nx, ny, nz_tot;              /* DOMAIN Nx, Ny, Nz                      */
  double L_x, L_y, L_z, z_i;
  double u_star, vonk, zo, dt;
  int sgs_model, cs_count, dyn_init, ifilter;
  int lbc_mom, ubc_mom;
  int molec;
  double nu_molec, ubot, utop;
  int use_mean_p_force, eval_mean_p_force;
  double mean_p_force_x, mean_p_force_y;
  int initu;                       /* restart semantics (initial.f90:98-106) */
  int precision;                   /* LESGO_FP64, LESGO_MIXED, LESGO_FP64_DW */
  /* actuator-disk turbines (TURBINES block); n_turbines = 0 disables */
  int n_turbines;
  const lesgo_turbine_t* turbines;
  double alpha1, alpha2, filter_cutoff, T_avg_dim;
  int adm_correction;
  /* time step chosen every step from the CFL number (cfl_util.f90:70-111,
   * main.f90:135-144); dt is then the step before the first one */
  int use_cfl_dt;
  double cfl;
} lesgo_params_t;

/* The run-control values of lesgo.conf that lesgo_params_t does not carry
 * (param.f90:100-240): read by lesgo_gpu_read_conf for the caller's loop. */
typedef struct {
  int nproc, uniform_spacing, wall_damp_exp, sgs;
  double Co;
  int nsteps, runtime, use_cfl_dt;
  double cfl;
  int cumulative_time, inilag;
  int wbase, nenergy, lag_cfl_count, checkpoint_data, checkpoint_nskip;
  int tavg_calc, tavg_nstart, tavg_nend, tavg_nskip;
  /* TURBINES dyn_theta1, dyn_theta2, dyn_Ct_prime: the schedules to read
   * with lesgo_gpu_read_turbine_schedule and set per handle */
  int dyn_theta1, dyn_theta2, dyn_ct_prime;
} lesgo_run_t;

typedef struct lesgo_handle lesgo_handle_t;

/* Fill *p with lesgo.conf defaults of the half-channel case (lbc_mom=2,
 * ubc_mom=0, sgs_model=5, cs_count=5, dyn_init=100, zo=1e-4, dt=2e-4). */
int lesgo_gpu_params_default(lesgo_params_t* p);

/* Create / destroy a solver on the current CUDA device.  Replaces
 * initialize() device-side parts: sim_param_init, sgs_param_init,
 * init_fft, test_filter_init, grid%build, turbines_init
 * (initialize.f90:21-202). */
int lesgo_gpu_create(const lesgo_params_t* p, lesgo_handle_t** h);
int lesgo_gpu_destroy(lesgo_handle_t* h);
const char* lesgo_gpu_last_error(const lesgo_handle_t* h);

/* nz (= Nz+1), ld, lh, nx2, ny2 of the handle. */
int lesgo_gpu_dims(const lesgo_handle_t* h, int* nz, int* ld, int* lh, int* nx2, int* ny2);

/* Copy planes lbz..nzhi of a Fortran (ld, ny, lbz:nzhi) FP64 host array into
 * / out of the device field (levels outside 0..nz are rejected). */
int lesgo_gpu_set_field(lesgo_handle_t* h, int field, const double* host, int lbz, int nzhi);
int lesgo_gpu_get_field(lesgo_handle_t* h, int field, double* host, int lbz, int nzhi);
/* The same copies in stream order: they return once queued, behind the
 * handle's queued steps.  The host array must stay unchanged (set) and
 * unread (get) until lesgo_gpu_sync or a synchronous call on the handle;
 * with page-locked host memory the copies run while the host continues (and
 * while other handles' steps run on the device). */
int lesgo_gpu_set_field_async(lesgo_handle_t* h, int field, const double* host, int lbz, int nzhi);
int lesgo_gpu_get_field_async(lesgo_handle_t* h, int field, double* host, int lbz, int nzhi);

/* Field registry: remember a Fortran module array (c_loc) for a field, then
 * upload/download it on demand (init, checkpoint and output only). */
int lesgo_gpu_bind_field(lesgo_handle_t* h, int field, double* host, int lbz, int nzhi);
int lesgo_gpu_upload(lesgo_handle_t* h, int field);
int lesgo_gpu_download(lesgo_handle_t* h, int field);

/* Seeded half-channel initial condition: u = (1/0.4) ln(z/z0) (1 + 0.1 U),
 * v, w = 0.1 U with U = U(-1,1) from a counter-based hash of
 * (seed, field, i, j, k); w(1) = w(nz) = 0, u(nz) = u(nz-1), v(nz) = v(nz-1).
 * Stands in for ic_les (initial.f90:550-623). */
int lesgo_gpu_init_ic(lesgo_handle_t* h, uint64_t seed);

/* ---- stage entry points (one per reference subroutine) ----------------- */
/* derivatives.f90:166-211 */
int lesgo_gpu_filt_da(lesgo_handle_t* h, int f, int dfdx, int dfdy);
/* derivatives.f90:37-70, 73-106, 109-163 */
int lesgo_gpu_ddx(lesgo_handle_t* h, int f, int dfdx);
int lesgo_gpu_ddy(lesgo_handle_t* h, int f, int dfdy);
int lesgo_gpu_ddxy(lesgo_handle_t* h, int f, int dfdx, int dfdy);
/* derivatives.f90:214-264, 267-311 */
int lesgo_gpu_ddz_uv(lesgo_handle_t* h, int f, int dfdz);
int lesgo_gpu_ddz_w(lesgo_handle_t* h, int f, int dfdz);
/* test_filtermodule.f90:126-147: filter plane `level` of `f` in place */
int lesgo_gpu_test_filter(lesgo_handle_t* h, int f, int level);
/* wallstress.f90:21-257 */
int lesgo_gpu_wallstress(lesgo_handle_t* h);
/* sgs_stag_util.f90:33-464 (+ lagrange_Sdep.f90, interpolag_Sdep.f90);
 * uses the handle's step counters (jt, jt_total) */
int lesgo_gpu_sgs_stag(lesgo_handle_t* h);
/* divstress_uv.f90:21-85, divstress_w.f90:21-116 */
int lesgo_gpu_divstress_uv(lesgo_handle_t* h);
int lesgo_gpu_divstress_w(lesgo_handle_t* h);
/* convec.f90:21-333 */
int lesgo_gpu_convec(lesgo_handle_t* h);
/* forcing.f90:79-117 + turbines.f90:465-638 (fxa, fya, fza) */
int lesgo_gpu_turbines_forcing(lesgo_handle_t* h);
/* main.f90:143-157: advance jt/jt_total and save RHS into RHS_f */
int lesgo_gpu_begin_step(lesgo_handle_t* h);
/* main.f90:211-267: RHS = -RHS - divt (+ mean_p_force) (+ f_a) */
int lesgo_gpu_rhs_assemble(lesgo_handle_t* h);
/* main.f90:273-296: Euler first step + AB2 intermediate velocity */
int lesgo_gpu_ab2(lesgo_handle_t* h);
/* press_stag_array.f90:21-290 with tridag_array.f90:166-246 */
int lesgo_gpu_press_stag_array(lesgo_handle_t* h);
/* main.f90:321-326: RHS -= grad p */
int lesgo_gpu_rhs_sub_dp(lesgo_handle_t* h);
/* forcing.f90:149-244 */
int lesgo_gpu_project(lesgo_handle_t* h);
/* tridag_array.f90:166-246 on device arrays in the reference layout:
 * a, b, c real (lh, ny, n); r, u interleaved complex (2*lh, ny, n).  Solves
 * every kx < nx/2 column except the ky Nyquist row and kx = ky = 0 (whose
 * first level is still set to r/b).  Runs on the handle's stream and
 * returns when done; LESGO_ERR_NUMERIC on a zero pivot. */
int lesgo_gpu_tridag_array(lesgo_handle_t* h, const double* a, const double* b, const double* c,
                           const double* r, double* u, int lh, int ny, int n);
/* Allocation-free variant of lesgo_gpu_tridag_array.  No counterpart in
 * the reference.  For callers that cannot allocate device memory (they own
 * every buffer through their own pool, must not stall on cudaMalloc, or
 * hold no handle): it needs no handle and allocates nothing.  Scratch is a
 * fixed 16 MiB array inside the library (lh*ny*n <= 2^21 doubles; larger
 * problems get LESGO_ERR_ARG), held on every GPU that loads the library.
 * Never capturable: each call waits for its own result, so a call on a
 * capturing stream returns LESGO_ERR_ARG and queues nothing (the capture
 * stays intact).  Calls share the array: calls whose GPU work
 * overlaps race.  Launches on `stream` (NULL: default stream) and returns
 * when done; LESGO_ERR_NUMERIC on a zero pivot.  After a nonzero return,
 * lesgo_gpu_last_error(NULL) describes the failure; a successful call does
 * not clear that message, so read it only right after a failed call. */
int lesgo_gpu_tridag_array_noalloc(const double* a, const double* b, const double* c, const double* r,
                                   double* u, int lh, int ny, int n, void* stream);

/* ---- fused time loop ---------------------------------------------------- */
/* Advance nsteps full time steps (main.f90:130-344) with fused kernels and
 * CUDA-graph replay; identical in meaning to calling the stage entry points
 * in the reference order. */
int lesgo_gpu_step(lesgo_handle_t* h, int nsteps);
/* Block until all queued work of the handle is done; reports a zero pivot
 * met by the tridiagonal solve since the last check as LESGO_ERR_NUMERIC. */
int lesgo_gpu_sync(lesgo_handle_t* h);

/* Diagnostics as device reductions: rmsdiv (rmsdiv.f90:21-60), kinetic
 * energy (io.f90:99-141), max CFL (cfl_util.f90:35-64) and the plane-mean
 * bottom wall stress (functions.f90:882-905).  Any pointer may be NULL. */
int lesgo_gpu_diag(lesgo_handle_t* h, double* rmsdiv, double* ke, double* cfl, double* tau_bot);

/* Step counters (jt, jt_total) of the handle. */
int lesgo_gpu_counters(const lesgo_handle_t* h, int* jt, int* jt_total);

/* Per-turbine disk velocity u_d_T, thrust f_n and power P = -f_n u_d_T
 * (turbines.f90:576-588) after the last turbines_forcing. */
int lesgo_gpu_turbine_state(lesgo_handle_t* h, double* u_d_T, double* f_n, double* power, int n);

/* Number of this library's kernel launches issued by one fused step of the
 * given kind (0: normal step, 1: step with the dynamic SGS update). */
int lesgo_gpu_launches_per_step(const lesgo_handle_t* h, int with_sgs_update);

/* ---- batches (no reference counterpart: the reference runs one instance
 * per MPI job) ------------------------------------------------------------
 * A batch handle holds `capacity` slots of one grid size; every kernel of a
 * step processes all active instances in one launch.  Instances have their
 * own roughness length, IC seed, actuator disks and step counters; they
 * share the other parameters of `p` (whose zo / turbines are ignored here).
 * The stage entry points and lesgo_gpu_step act on every active instance;
 * per-instance access goes through the *_inst calls with the id from
 * lesgo_gpu_batch_add.  Removing an instance moves the last one into its
 * slot (ids stay valid). */
int lesgo_gpu_batch_create(const lesgo_params_t* p, int capacity, lesgo_handle_t** h);
int lesgo_gpu_batch_add(lesgo_handle_t* h, double zo, uint64_t seed, int n_turbines,
                        const lesgo_turbine_t* turbines, int* id);
int lesgo_gpu_batch_remove(lesgo_handle_t* h, int id);
int lesgo_gpu_batch_size(const lesgo_handle_t* h, int* active, int* capacity);
int lesgo_gpu_set_field_inst(lesgo_handle_t* h, int id, int field, const double* host, int lbz, int nzhi);
int lesgo_gpu_get_field_inst(lesgo_handle_t* h, int id, int field, double* host, int lbz, int nzhi);
int lesgo_gpu_set_field_inst_async(lesgo_handle_t* h, int id, int field, const double* host, int lbz, int nzhi);
int lesgo_gpu_get_field_inst_async(lesgo_handle_t* h, int id, int field, double* host, int lbz, int nzhi);
int lesgo_gpu_diag_inst(lesgo_handle_t* h, int id, double* rmsdiv, double* ke, double* cfl, double* tau_bot);
int lesgo_gpu_counters_inst(lesgo_handle_t* h, int id, int* jt, int* jt_total);
int lesgo_gpu_turbine_state_inst(lesgo_handle_t* h, int id, double* u_d_T, double* f_n, double* power, int n);
/* Device bytes a handle of this grid and capacity allocates (admission). */
int lesgo_gpu_footprint(const lesgo_params_t* p, int capacity, long long* bytes);

/* ---- diagnostics log (main.f90:359-436: the wbase / nenergy output) -----
 * After every step whose jt_total is a multiple of `every`, each instance
 * appends one row (jt_total, total_time, rmsdiv, ke, cfl, tau_wall_bot)
 * computed on the device, with no host synchronisation, to a ring of
 * `capacity` rows.  lesgo_gpu_diag_log_read copies the newest min(rows
 * written, capacity, maxrows) rows, oldest first, 6 doubles each.
 * lesgo_gpu_diag_log_sample applies the schedule once now (drop-in callers). */
int lesgo_gpu_diag_log_config(lesgo_handle_t* h, int every, int capacity);
int lesgo_gpu_diag_log_sample(lesgo_handle_t* h);
int lesgo_gpu_diag_log_read(lesgo_handle_t* h, int id, double* rows, int maxrows, int* nrows);

/* ---- time-averaging statistics (time_average.f90; schedule io.f90:557-580)
 * After every step, per instance: steps jt_total in [nstart, nend] add dt to
 * the pending weight; a step with (jt_total - nstart) % nskip == 0 starts the
 * sums (first time, tavg%init) or adds the fields times the pending weight
 * (tavg%compute).  Sums are FP64 on the device, levels 1..nz.  `which`
 * selects an average: 0 u, 1 v, 2 w, 3 u_w, 4 v_w, 5 w_uv, 6 u2, 7 v2, 8 w2,
 * 9 uv, 10 uw, 11 vw, 12 txx, 13 tyy, 14 tzz, 15 txy, 16 txz, 17 tyz,
 * 18 p (real pressure), 19 fx, 20 fy, 21 fz, 22 cs_opt2, 23 vortx, 24 vorty,
 * 25 vortz; or a Reynolds stress (time_average.f90:616-629): 26 up2, 27 vp2,
 * 28 wp2, 29 upvp, 30 upwp, 31 vpwp.  Fields are (ld, ny, lbz..nzhi) like
 * lesgo_gpu_get_field. */
int lesgo_gpu_tavg_config(lesgo_handle_t* h, int nstart, int nend, int nskip);
/* Apply the schedule once now (for callers driving the stage entry points). */
int lesgo_gpu_tavg_sample(lesgo_handle_t* h);
int lesgo_gpu_tavg_get(lesgo_handle_t* h, int which, double* host, int lbz, int nzhi);
int lesgo_gpu_tavg_get_inst(lesgo_handle_t* h, int id, int which, double* host, int lbz, int nzhi);
/* Plane (x-y) mean of an average at levels 0..nz: prof[n >= nz+1]. */
int lesgo_gpu_tavg_profile(lesgo_handle_t* h, int which, double* prof, int n);
int lesgo_gpu_tavg_profile_inst(lesgo_handle_t* h, int id, int which, double* prof, int n);
/* tavg%total_time of instance id (id < 0: the handle's single instance). */
int lesgo_gpu_tavg_total_time(lesgo_handle_t* h, int id, double* total_time);

/* ---- configuration (input_util.f90:54-1023 read_input_conf; turbine
 * placement turbines.f90:740-866) -----------------------------------------
 * Reads <path>lesgo.conf into *p (reference defaults for absent keys) and
 * *run.  with_turbines != 0 parses the TURBINES block (else it is skipped
 * like a build without turbines) and places the disks into turbines[0..max):
 * p->turbines points there and p->n_turbines counts them; read_param reads
 * <path>input_turbines/param.dat.  Host only (no device is touched).
 * Malformed files: LESGO_ERR_ARG with file:line in lesgo_gpu_last_error(NULL);
 * settings whose physics this library leaves out (coriolis_forcing,
 * use_sponge, inflow_type, use_random_force, sgs = .false., rotating
 * turbines): LESGO_ERR_UNSUPPORTED.  Time-varying yaw, tilt and Ct' are
 * reported in run->dyn_*.  `log` (may be NULL) receives
 * the reference's notes on unused blocks and keys. */
int lesgo_gpu_read_conf(const char* path, int with_turbines, lesgo_params_t* p, lesgo_run_t* run,
                        lesgo_turbine_t* turbines, int max_turbines, char* log, int loglen);

/* ---- turbine control schedules (turbines.f90:500-515; files read by
 * read_control_files, turbines.f90:872-931) ---------------------------------
 * which: 0 yaw theta1, 1 tilt theta2 (degrees), 2 Ct'.  `rows` holds nt
 * rows of 1 + n_turbines values, as the lines of input_turbines/theta1.dat:
 * the dimensional time, then one value per turbine of the instance.  Every
 * step each turbine takes the value linearly interpolated at the step's
 * total_time_dim (binary_search + linear_interp, functions.f90:712-860;
 * constant beyond the first and last rows).  A yaw or tilt schedule
 * re-evaluates the actuator-disk nodes and indicator values on the device
 * each step (turbines_nodes, turbines.f90:275-462).  nt = 0 removes the
 * schedule.  Times must not decrease; the instance must have turbines. */
int lesgo_gpu_turbine_schedule(lesgo_handle_t* h, int which, int nt, const double* rows);
int lesgo_gpu_turbine_schedule_inst(lesgo_handle_t* h, int id, int which, int nt, const double* rows);
/* Read <path>input_turbines/theta1.dat (which 0), theta2.dat (1) or
 * Ct_prime.dat (2) for n_turbines disks into rows (max_rows rows of
 * 1 + n_turbines values); *nt receives the row count.  Host only. */
int lesgo_gpu_read_turbine_schedule(const char* path, int which, int n_turbines, double* rows, int max_rows,
                                    int* nt);
/* Current yaw and tilt (degrees) and Ct' of the instance's turbines, as
 * the last step used them (the static values before any step). */
int lesgo_gpu_turbine_controls(lesgo_handle_t* h, int id, double* theta1, double* theta2, double* ct_prime, int n);

/* ---- checkpoint / restart (io.f90:1173-1267 checkpoint; initial.f90:20-380
 * and io.f90:60-96 restart) ------------------------------------------------
 * `path` is a prefix like the reference's `path` (a directory with its
 * trailing '/').  Writes <path>vel.out (one Fortran unformatted sequential
 * record: u, v, w, RHSx, RHSy, RHSz, Cs_opt2, F_LM, F_MM, F_QN, F_NN, each
 * (ld, ny, 1:nz) FP64), <path>grid.out, <path>total_time.dat and, when time
 * averaging has started, <path>tavg.out.  mpi_names != 0 names the per-rank
 * files like an MPI run of one rank (vel.out.c0, tavg.out.c0). */
int lesgo_gpu_checkpoint_write(lesgo_handle_t* h, const char* path, int mpi_names);
int lesgo_gpu_checkpoint_write_inst(lesgo_handle_t* h, int id, const char* path, int mpi_names);
/* Restart from <path>vel.out (or vel.out.c0; vel.out.c<n> per rank of an MPI
 * checkpoint).  Same grid and one rank (grid.out): every field is taken and
 * the run continues as initu (no Euler first step, no Lagrangian
 * initialisation); *same_grid = 1.  Otherwise u, v, w are interpolated onto
 * this grid (ic_interp) and the other fields start at zero; *same_grid = 0.
 * total_time.dat, if present, sets jt_total and total_time (jt restarts at
 * 0).  With time averaging configured, tavg.out's sums are taken up at the
 * first sample step.  Missing or malformed files: LESGO_ERR_ARG. */
int lesgo_gpu_checkpoint_read(lesgo_handle_t* h, const char* path, int* same_grid);
int lesgo_gpu_checkpoint_read_inst(lesgo_handle_t* h, int id, const char* path, int* same_grid);
/* total_time of instance id (id < 0: the handle's single instance). */
int lesgo_gpu_sim_time(lesgo_handle_t* h, int id, double* total_time);
/* dt of instance id's last step (with use_cfl_dt the one cfl_util.f90:70-111
 * chose on the device; before the first step the input dt). */
int lesgo_gpu_time_step(lesgo_handle_t* h, int id, double* dt);

/* ---- tile-shape autotuner (no reference counterpart) ----------------------
 * Picks the tile shapes of the transform passes (complex values per block of
 * the x passes, shared-memory bytes per block of the y passes) by timing the
 * handle's own fused step at every candidate, and returns them.  The fields,
 * step constants and disk states are copied aside on the device first and
 * put back after, so the simulation state is unchanged (tile shapes do not
 * change results); without memory for that copy the passes are timed alone
 * on scratch buffers.  Call it once after the instances are in place. */
int lesgo_gpu_autotune(lesgo_handle_t* h, int* xtarget, int* ybudget);

/* ---- instrumentation (no reference counterpart; the reference only
 * prints wall-clock times, main.f90:359-436) --------------------------- */
/* enable != 0: run steps eagerly (no graph replay) with a CUDA event pair
 * on the handle's stream around every kernel; resets the records. */
int lesgo_gpu_profile(lesgo_handle_t* h, int enable);
/* JSON object {"kernel": [launches, total_ms, algorithmic_bytes], ...}. */
int lesgo_gpu_profile_report(lesgo_handle_t* h, char* buf, int buflen);
/* The cudaStream_t the handle launches on (for events recorded by callers). */
int lesgo_gpu_get_stream(const lesgo_handle_t* h, void** stream);

#ifdef __cplusplus
}
#endif
#endif /* LESGO_GPU_H */
