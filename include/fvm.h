/*
 * fvm.h -- C-ABI of the GB300 time step of the fractional 4-step incompressible
 * Navier-Stokes finite-volume solver on a curvilinear cylinder O-grid.
 *
 * Drop-in boundary.  The reference (Fortran 90, cylinder/cylinder_v3.0.3_AF_
 * original 4step_face_nl/) drives one time step from PROGRAM MAIN
 * (Main.f90:48-114) through argument-less subroutines sharing module globals
 * (comdat_shared.f90).  This library owns those globals on the GPU: a context
 * holds every field, metric and scratch array in device memory, and each entry
 * point below replaces one call point of the reference's time loop.  All
 * functions take plain pointers and sizes, are callable from Fortran through
 * ISO_C_BINDING (BIND(C)), and return an int status (FVM_OK = 0) -- they never
 * abort.  fvm_last_error() gives the message of the last failure.
 *
 * Array layout: every field array is the reference's Fortran array (0:NI,0:NJ)
 * of DOUBLE PRECISION, element (I,J) at index I + (NI+1)*J (I radial, I=0 the
 * wall ghost, I=NI the far-field ghost; J circumferential, J=0 and J=NJ the
 * branch-cut ghosts).  Node coordinates XG, YG use the same (NI+1)*(NJ+1)
 * storage with I = 1..NI, J = 1..NJ valid.
 *
 * Threading: one context = one CUDA stream on one device.  Distinct contexts
 * may be used from distinct host threads; one context must not be used by two
 * threads at once.  Host arrays are only read or written during the call that
 * receives them; no pointer is retained.
 */
#ifndef FVM_GB300_H
#define FVM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FVM_OK = 0,
    FVM_ERR_ARG = 1,      /* invalid argument or call order */
    FVM_ERR_CUDA = 2,     /* CUDA runtime error (message in fvm_last_error) */
    FVM_ERR_NOCONV = 3,   /* Poisson sweep cap reached above tolerance (fields are valid) */
    FVM_ERR_TIMEOUT = 4,  /* a bounded device-side wait ran out */
    FVM_ERR_NAN = 5,      /* non-finite value detected in the step's coefficients */
    FVM_ERR_NOMEM = 6     /* device allocation failed */
};

enum { FVM_FP64 = 0, FVM_MIXED = 1 };       /* precision of the line sweeps */
enum { FVM_FIELD_U = 0, FVM_FIELD_V = 1, FVM_FIELD_T = 2 };

/* Run parameters.  The reference takes NI, NJ, NSWPP, RESIMAX, UIN, VIN, TIN,
 * T_WALL as compile-time PARAMETERs (comdat_param.f90:6-39) and RE, PR,
 * VEL_ROT, DTIME from standard input (Main.f90:23-36). */
typedef struct fvm_params {
    int ni, nj;            /* NI, NJ: node counts; cells 1..NI-1 x 1..NJ-1; NJ-1 must be even */
    double re, pr, dt, vel_rot;
    double uin, vin, tin, t_wall;
    double resimax;        /* Poisson scaled-L1 residual tolerance (RESIMAX) */
    int nswpp;             /* Poisson sweep cap (NSWPP) */
    int precision;         /* FVM_FP64 or FVM_MIXED */
    int thermal;           /* 1: advance the passive temperature (ITER_T) */
    int iter_t_bug;        /* 1: keep the reference's V in ITER_T's second cross term */
    int res_every;         /* FP64: evaluate the Poisson residual every k-th sweep (>=1) */
    int refine_sweeps;     /* MIXED: FP32 zebra sweeps per FP64 residual/refinement */
    int adi_refine;        /* MIXED: FP64 defect-correction passes per predictor line solve */
    int device;            /* CUDA device ordinal */
    int poisson_groups;    /* residual intervals per Poisson graph body (0: about 32 sweeps) */
    int poisson_host_loop; /* 1: the host replays the body until done (default; kernels stay visible
                              to profilers); 0: the loop ends on the device in a graph while-node */
    int dd_positional;     /* 1 (default): DIF and ITER_P add the cross term of cell (I-1,J-1) to
                              cell (I,J), zero on row/column 1, as the reference's whole-array DD
                              operand evaluates (dif.f90:15-23, iter_p.f90:27-30); 0: cell (I,J) */
    /* Line tiles (0 = automatic): warps per line group (1, 2 or 4) and elements per
       thread (1..4; also 6, 8, 12 with one warp, 6, 8 with two) of the radial lines
       (NI-1 unknowns: Poisson and first predictor factor) and of the circumferential
       lines (NJ-1 unknowns: second factor); 32 * warps * elements must cover the
       line.  Set both of a family or neither. */
    int tile_r_warps, tile_r_m, tile_t_warps, tile_t_m;
    /* MIXED, single context: FP32 correction sweeps of one refinement interval in
       one launch whose blocks keep their lines on chip and exchange only boundary
       lines (1, the default: lines per block chosen automatically; k >= 2, even:
       k lines per block; 0: one launch per zebra colour).  Same results bit for bit. */
    int poisson_resident;
    /* Resident sweeps: sweeps per exchange of boundary lines between blocks (0, the
       default: 2 where the layout allows it -- 4 lines per block, line groups of one
       or two warps, NJ-1 >= 12 -- else 1; 1; 2: required).  Two sweeps per exchange
       solve three more lines per block redundantly and halve the exchanges.  Same
       results bit for bit. */
    int resident_depth;
} fvm_params;

/* Per-step diagnostics of CALCCOEF (calccoef.f90:9-120) plus Poisson statistics. */
typedef struct fvm_coeffs {
    double time, cfl, cpb, cd, cl, cd_p, cd_v, cl_p, cl_v, nu;
    int sweeps;            /* Poisson sweeps of the last step */
    double resid;          /* last scaled residual of the last step */
} fvm_coeffs;

/* Defaults: the reference's PARAMETER values (comdat_param.f90:11-19), FP64. */
int fvm_default_params(fvm_params *p);

/* Context life cycle.  Replaces the module COMDAT_SHARED (comdat_shared.f90:38-162). */
int fvm_create(const fvm_params *p, struct fvm_ctx **ctx);
int fvm_destroy(struct fvm_ctx *ctx);
const char *fvm_last_error(const struct fvm_ctx *ctx);

/* GRID + METRIC (grid.f90:28-114, metric.f90:18-168) from node coordinates. */
int fvm_set_grid(struct fvm_ctx *ctx, const double *xg, const double *yg);
/* INIT (init.f90:17-137): uniform flow; du/dv (may be NULL) are added to the
 * interior of U and V before the boundary conditions. */
int fvm_init(struct fvm_ctx *ctx, const double *du, const double *dv);

/* Host <-> device copies of the time-step state (the RESTART.DAT contents,
 * writedata.f90:77-90).  Any pointer may be NULL to skip that array. */
int fvm_upload_state(struct fvm_ctx *ctx, const double *u, const double *v, const double *p,
                     const double *t, const double *nlx, const double *nly, const double *adv);
int fvm_download_state(struct fvm_ctx *ctx, double *u, double *v, double *p, double *t,
                       double *nlx, double *nly, double *adv);
/* Named access to any context array (names as in comdat_shared.f90, e.g.
 * "U", "DJAC", "S_U", "UE"); out/in hold (NI+1)*(NJ+1) doubles. */
int fvm_get_array(struct fvm_ctx *ctx, const char *name, double *out);
int fvm_set_array(struct fvm_ctx *ctx, const char *name, const double *in);
int fvm_set_time(struct fvm_ctx *ctx, double rtime, int niter_time);
/* Wall controls (no reference counterpart beyond VEL_ROT): rotation rate omega
 * (the reference's VEL_ROT, bcu.f90:13) and a wall-normal blowing speed per wall
 * cell, blow[J-1] for J=1..NJ-1 (NULL: none).  The wall velocity of cell J is
 * omega*(-sin th, cos th) + blow*(cos th, sin th) with th = THETA(0,J), and the
 * wall face flux UW(1,J) (zero in contra_vel.f90:125) becomes blow times the face
 * value of J*(xi_x cos th + xi_y sin th).  With blow = 0 the step is the
 * reference's. */
int fvm_set_controls(struct fvm_ctx *ctx, double omega, const double *blow);

/* Post-processing phase (calccoef.f90:156-190, post_process.f90:8-62,
 * calc_vor.f90:14-58).
 * fvm_post_begin: POST_PROCESS with IPOST=0 -- NITER_POS=0, TOGGLE=1, the sums
 *   cleared; from the next step on, every CALCCOEF (fvm_step, fvm_calccoef)
 *   runs CALC_VOR, the lift-extremum test (ST = 1/(t - t two extrema ago),
 *   CL_AMP = |CL - CL at the last extremum|/2), adds U,V,P,T,VOR to their time
 *   sums on the device and Nu,Cd,Cl,St,Cpb,CL_AMP and the squared deviations of
 *   Cd, Cl from their running means to host sums.
 * fvm_post_get: the record CALCCOEF appends to POST_NU_CD_CL.PLT for the last
 *   step (calccoef.f90:186-188).
 * fvm_post_final: POST_PROCESS with IPOST=1 -- the averages (the
 *   TIME_AVERAGED_RESULTS.DAT record) and the time-averaged fields of
 *   TIME-AVERAGED FIELD.PLT into host arrays (any may be NULL).  Unlike the
 *   reference, which overwrites its state with the averages at the end of its
 *   run, the state is left unchanged.
 * fvm_post_end: averaging off.
 * fvm_calc_vor: CALC_VOR into the array "VOR" (fvm_get_array).  The sums are
 *   readable as "U_TA", "V_TA", "P_TA", "T_TA", "VOR_TA" once averaging began. */
typedef struct fvm_post {
    double time, nu, cd, cl, cl_amp, cpb, st, rms_cd, rms_cl;
    double st_last, cl_amp_last;   /* ST and CL_AMP of the last extremum pair */
    int niter;                     /* NITER_POS: steps averaged */
} fvm_post;

int fvm_post_begin(struct fvm_ctx *ctx);
int fvm_post_get(struct fvm_ctx *ctx, fvm_post *out);
int fvm_post_final(struct fvm_ctx *ctx, fvm_post *out, double *u, double *v, double *p, double *t,
                   double *vor);
int fvm_post_end(struct fvm_ctx *ctx);
int fvm_calc_vor(struct fvm_ctx *ctx);

/* Discrete adjoint (no reference counterpart).  From the current state, runs
 * `window` steps (the state advances, as fvm_step would) and returns
 * J = mean over those steps of the drag coefficient CALCCOEF reports, with its
 * exact gradient for the discrete step (Poisson taken as converged) with respect
 * to the rotation rate (dJ_domega) and the NJ-1 blowing speeds (dJ_dblow), the
 * controls held fixed over the window.  The state is checkpointed every `ckpt`
 * steps and each segment recomputed for the reverse pass.  Any output may be
 * NULL.  Returns FVM_ERR_NOCONV if a forward step hit its sweep cap. */
int fvm_adjoint_drag_grad(struct fvm_ctx *ctx, int window, int ckpt, double *J, double *dJ_domega,
                          double *dJ_dblow);
/* Transpose of one step at the current state (the state is left unchanged): the
 * five host arrays (U, V, P, NLX, NLY adjoints, full-array storage) hold on
 * entry the adjoint of the state after the step and on exit that of the state
 * before it; dctrl (may be NULL) receives 1 + (NJ-1) control adjoints
 * (rotation, then blowing). */
int fvm_adjoint_vjp(struct fvm_ctx *ctx, double *lu, double *lv, double *lp, double *lnlx, double *lnly,
                    double *dctrl);

/* One call point each of the reference time loop (Main.f90:48-114). */
int fvm_begin_step(struct fvm_ctx *ctx);   /* Main.f90:48-54: time advance, U_N=U, V_N=V, T_N=T */
int fvm_contra_vel(struct fvm_ctx *ctx);   /* CONTRA_VEL, contra_vel.f90:9-21,125 */
int fvm_nl(struct fvm_ctx *ctx, int field);   /* NL(U_N,NLX) etc., nl.f90:21-27 (shifts *_NM1 first) */
int fvm_dif(struct fvm_ctx *ctx, int field);  /* DIF(U_N,DIFX) etc., dif.f90 + dif_diagonal.f90 */
int fvm_p_source(struct fvm_ctx *ctx);     /* P_SOURCE, p_source.f90:9-27 */
int fvm_iter_u(struct fvm_ctx *ctx);       /* ITER_U, iter_u.f90:13-119 (with BCU) */
int fvm_iter_v(struct fvm_ctx *ctx);       /* ITER_V, iter_v.f90 (with BCV) */
int fvm_remove_grad(struct fvm_ctx *ctx);  /* Main.f90:80-87: u^ = u* - dt S/J, BCU, BCV */
/* Main.f90:91-93: CONTRA_VEL, ITER_P (iter_p.f90:12-51 with LISOLV and BCP), BCP.
 * resid/sweeps may be NULL.  Returns FVM_ERR_NOCONV if the cap was reached. */
int fvm_iter_p(struct fvm_ctx *ctx, double *resid, int *sweeps);
int fvm_correct(struct fvm_ctx *ctx);      /* Main.f90:97-107: P_SOURCE, u += dt S/J, BCU, BCV */
int fvm_iter_t(struct fvm_ctx *ctx);       /* Main.f90:110-111: ITER_T (iter_T.f90) and BCT */
int fvm_calccoef(struct fvm_ctx *ctx, fvm_coeffs *out);  /* CALCCOEF, calccoef.f90:9-120 */

/* nsteps complete time steps (Main.f90:48-114 without file output), state kept
 * on the device.  out (may be NULL) receives the last step's coefficients.
 * Returns FVM_ERR_NOCONV if any step hit the sweep cap (the run continues, as in
 * the reference). */
int fvm_step(struct fvm_ctx *ctx, int nsteps, fvm_coeffs *out);
/* Per-step coefficient history of the last fvm_step call: n entries copied. */
int fvm_history(struct fvm_ctx *ctx, fvm_coeffs *out, int n);

/* Block until all work queued on the context's stream has finished. */
int fvm_synchronize(struct fvm_ctx *ctx);

/* Instrumentation (no reference counterpart; used by benchmarks).  The CUDA
 * stream of the context (a cudaStream_t), and counters accumulated since the last
 * reset: CUDA-event time of the sweep-kernel replays of fvm_time_sweeps and
 * their launch count, every kernel the context launched (device-side loop
 * iterations included), Poisson sweeps and time steps. */
typedef struct fvm_timing {
    double sweep_span_ms;
    long long sweep_span_launches;
    long long kernel_launches;
    long long sweeps;
    long long steps;
} fvm_timing;
int fvm_get_stream(struct fvm_ctx *ctx, void **stream);
int fvm_timing_reset(struct fvm_ctx *ctx);
int fvm_get_timing(struct fvm_ctx *ctx, fvm_timing *out);
/* Replays `sweeps` zebra sweeps of the Poisson sweep kernels of the context's
 * precision (touching only scratch arrays, the state is unchanged) in a graph
 * bracketed by CUDA events on the context's stream.  ms_per_launch: average time
 * per zebra colour (the per-colour path launches once per colour; the resident
 * path runs all sweeps in one launch, reported as 1 in *launches, and the figure
 * is its time divided by 2*sweeps). */
int fvm_time_sweeps(struct fvm_ctx *ctx, int sweeps, double *ms_per_launch, long long *launches);
/* Check of the bounded waits of the resident sweeps (MIXED contexts using them):
 * four sweeps on scratch arrays with exchange tags that no block publishes, so
 * every wait for a neighbouring block runs out after max_polls polls (1 .. 2^24).
 * Returns FVM_ERR_TIMEOUT when the kernel reported it, as a step would; the
 * state is unchanged and the exchange state cleared, so the context stays usable.
 * FVM_ERR_ARG if the context does not use the resident path. */
int fvm_resident_wait_test(struct fvm_ctx *ctx, int max_polls);
/* Layout of the resident Poisson sweeps the context chose: lines per block (0: the
 * per-colour path), blocks, and sweeps per exchange of boundary lines (1 or 2). */
int fvm_resident_info(struct fvm_ctx *ctx, int *lines_per_block, int *blocks, int *sweeps_per_exchange);

/* Allocation-free scaled residual of the pressure equation.  No counterpart in
 * the reference: it serves callers that cannot allocate device memory (code
 * recording a CUDA graph, where cudaMalloc is not allowed, or a host program whose
 * device memory belongs to a pool or framework allocator).  It needs no context
 * and allocates nothing; its only scratch is a fixed 32 KiB static device array
 * that every GPU loading the library keeps until exit.
 *   p, su, ap, ae, aw, an, as: caller-owned DEVICE arrays in the field layout above
 *   (P with its ghost cells, the right-hand side SU and the five coefficients);
 *   resid: caller-owned DEVICE pointer receiving sum|r| / sum|AP*P| over the
 *   interior, r = AE P(I+1) + AW P(I-1) + AN P(J+1) + AS P(J-1) + SU - AP P with
 *   J+1 / J-1 taken through the periodic branch cut; stream: a cudaStream_t (NULL:
 *   the default stream).  The call is asynchronous on that stream.
 * Limit: (NI-1)*(NJ-1) <= 1,048,576 interior cells, else FVM_ERR_ARG.  The first
 * call on a device resolves the scratch address (once per device, with that device
 * current) and should come before any stream capture.  All calls share the
 * scratch, so calls that may overlap on the GPU (other streams, other host threads)
 * race and must be serialised by the caller.  The resolved address is kept until
 * the process exits: do not call this entry point after a cudaDeviceReset of that
 * device (the scratch it would use is no longer mapped). */
int fvm_poisson_residual_static(int ni, int nj, const double *p, const double *su, const double *ap,
                                const double *ae, const double *aw, const double *an, const double *as,
                                double *resid, void *stream);

/* ---------------------------------------------------------------------------
 * Batches: many independent cases (different grids, Re, Pr, dt, rotation,
 * tolerances) advanced together, each sub-step one launch over all cases and the
 * whole time step one CUDA graph (the Poisson loop runs on the device until the
 * last case has converged or reached its cap).  No reference counterpart: the
 * reference runs one case per process (Main.f90:40-118 once per run).
 * --------------------------------------------------------------------------- */
struct fvm_batch;
/* params: ncases entries.  precision, thermal, iter_t_bug, res_every,
 * refine_sweeps, device, poisson_groups and the tile fields must agree; tiles left
 * at 0 become the automatic tile of the longest line of the batch. */
int fvm_batch_create(int ncases, const fvm_params *params, struct fvm_batch **out);
int fvm_batch_destroy(struct fvm_batch *b);
const char *fvm_batch_last_error(const struct fvm_batch *b);
/* The context of case k, owned by the batch: set it up with fvm_set_grid and
 * fvm_init / fvm_upload_state, read it with fvm_get_array / fvm_download_state. */
int fvm_batch_case(struct fvm_batch *b, int k, struct fvm_ctx **ctx);
/* Line tiles shared by the cases: {radial warps, radial elements per thread,
 * circumferential warps, circumferential elements per thread}. */
int fvm_batch_tiles(const struct fvm_batch *b, int *tiles);
int fvm_batch_set_tiles(struct fvm_batch *b, const int *tiles);
/* Times every tile that covers the batch's lines on the batch itself (`sweeps`
 * replays of the batched Poisson sweep for the radial family, of the batched
 * circumferential predictor sweep for the other) and keeps the fastest.  Needs
 * every case's grid; the flow state is left unchanged.  tiles (4 ints) and ms
 * (2 doubles: best time per sweep of each family) may be NULL. */
int fvm_batch_autotune(struct fvm_batch *b, int sweeps, int *tiles, double *ms);
/* Average time of one batched Poisson sweep (both colours, state unchanged). */
int fvm_batch_time_sweeps(struct fvm_batch *b, int sweeps, double *ms_per_sweep);
/* nsteps time steps of every case.  out (may be NULL) receives nsteps*ncases
 * records, step-major (out[s*ncases + k]); each case's fvm_history holds its own.
 * Returns FVM_ERR_NOCONV if any case hit its sweep cap. */
int fvm_batch_step(struct fvm_batch *b, int nsteps, fvm_coeffs *out);
int fvm_batch_get_timing(const struct fvm_batch *b, fvm_timing *out);

#ifdef __cplusplus
}
#endif
#endif
