/*
 * fvm_oracle.h -- CPU restatement of the reference's 2-D fractional 4-step
 * incompressible Navier-Stokes time step (cylinder O-grid), used ONLY as test
 * infrastructure: the parity tests, the smoke check and the CPU-baseline leg of
 * the benchmark call it as the checker.  The product (the CUDA library behind
 * include/fvm.h) never links or calls this code.
 *
 * Reference: cylinder/cylinder_v3.0.3_AF_original 4step_face_nl/ (Fortran 90).
 * The reference cannot be compiled here (no Fortran compiler on either machine)
 * and ships no tests or golden vectors.  The restatement is pinned instead by
 * executing the reference's own source files: tests/golden/make_golden.py runs
 * them through a Fortran-subset interpreter (tests/golden/ftn_interp.py) on small
 * grids and commits U, V, P, T, NLX, NLY, ADV and every coefficient record as
 * fixtures; ORC_FAITHFUL with dd_positional=1 reproduces them (tests compare at
 * 1e-12 relative L2 and 1e-11 on the coefficients).
 *
 * Arrays follow the reference layout: Fortran order (0:NI, 0:NJ), element
 * (i, j) at i + (NI+1)*j, I radial (wall ghost i=0, far-field ghost i=NI),
 * J circumferential and periodic through the branch cut (ghost rows j=0, j=NJ).
 * Node arrays XG/YG use the same (NI+1)*(NJ+1) storage, valid for
 * i = 1..NI, j = 1..NJ.
 */
#ifndef FVM_ORACLE_H
#define FVM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Ordering of the line sweeps.
 *  ORC_FAITHFUL : the reference's lexicographic line Gauss-Seidel order, lagged
 *                 ghost rows across the branch cut (iter_u.f90:50-119,
 *                 lisolv.f90:18-33).
 *  ORC_GPU      : the order the GPU implements: zebra (odd lines, then even
 *                 lines) in every line sweep, periodic index wrap across the
 *                 branch cut inside sweeps and residuals, and cyclic tridiagonal
 *                 solves for the circumferential lines of the momentum/thermal
 *                 predictor.  Everything else is identical to ORC_FAITHFUL. */
enum { ORC_FAITHFUL = 0, ORC_GPU = 1 };

typedef struct {
    int ni, nj;          /* reference NI, NJ (node counts); cells 1..NI-1 x 1..NJ-1 */
    double re, pr, dt, vel_rot;
    double uin, vin, tin, t_wall;
    double resimax;      /* Poisson scaled-L1 tolerance (reference RESIMAX) */
    int nswpp;           /* Poisson sweep cap (reference NSWPP) */
    int order;           /* ORC_FAITHFUL or ORC_GPU */
    int iter_t_bug;      /* 1: second-sweep cross term of ITER_T built from V (iter_T.f90:89-95) */
    int thermal;         /* 1: advance the passive temperature (ITER_T + BCT) */
    int res_every;       /* ORC_GPU: residual evaluated every k-th sweep (>=1) */
    int dd_positional;   /* 1: DIF and ITER_P add the cross term of cell (I-1,J-1), as the
                            reference's whole-array DD operand in an interior-section
                            expression evaluates (dif.f90:15-23, iter_p.f90:27-30);
                            0: the cross term of cell (I,J) */
} orc_params;

typedef struct {
    double time, cfl, cpb, cd, cl, cd_p, cd_v, cl_p, cl_v, nu;
    int sweeps;          /* Poisson sweeps of the last step */
    double resid;        /* final scaled residual of the last step */
} orc_coeffs;

/* Record of the post-processing phase: what CALCCOEF appends to
 * POST_NU_CD_CL.PLT after each step (calccoef.f90:186-188) -- time averages of
 * Nu, Cd, Cl, the lift half-amplitude, Cpb and St, and the rms of Cd and Cl about
 * the running means -- plus ST and CL_AMP of the last detected extremum pair. */
typedef struct {
    double time, nu, cd, cl, cl_amp, cpb, st, rms_cd, rms_cl;
    double st_last, cl_amp_last;
    int niter;           /* NITER_POS: steps averaged */
} orc_post;

typedef struct orc orc;

orc *orc_create(const orc_params *p);
void orc_destroy(orc *o);
/* GRID (cell centres, ghost re-positioning) + METRIC + the geometry part of INIT.
 * xg, yg: node coordinates, (NI+1)*(NJ+1) storage, i=1..NI, j=1..NJ used. */
int orc_set_grid(orc *o, const double *xg, const double *yg);
/* INIT: uniform flow, optional interior perturbation added before the boundary
 * conditions (du, dv may be NULL; full-array storage). */
int orc_init(orc *o, const double *du, const double *dv);
/* Full time step(s), Main.f90:48-114. */
int orc_step(orc *o, int nsteps);
const orc_coeffs *orc_last_coeffs(const orc *o);

/* Sub-steps in reference call order (for sub-step parity tests). */
void orc_begin_step(orc *o);      /* Main.f90:48-54 */
void orc_contra_vel(orc *o);      /* contra_vel.f90 */
void orc_explicit(orc *o);        /* Main.f90:61-74: NL x3, DIF x3, P_SOURCE */
void orc_iter_u(orc *o);
void orc_iter_v(orc *o);
void orc_remove_grad(orc *o);     /* Main.f90:80-87 */
int  orc_iter_p(orc *o);          /* Main.f90:91-93: CONTRA_VEL, ITER_P, BCP; returns sweeps */
void orc_correct(orc *o);         /* Main.f90:97-107 */
void orc_iter_t(orc *o);          /* Main.f90:110-111 */
void orc_calccoef(orc *o);        /* calccoef.f90 */

/* Wall controls, no reference counterpart: rotation rate omega (VEL_ROT) and a
 * wall-normal blowing speed per wall cell (blow[J-1] for J=1..NJ-1; NULL = 0),
 * entering the wall velocity of BCU/BCV and the wall face flux UW(1,J). */
void orc_set_controls(orc *o, double omega, const double *blow);

/* Post-processing (no effect on the flow).
 * orc_post_begin: POST_PROCESS with IPOST=0 (post_process.f90:8-16): NITER_POS=0,
 *   TOGGLE=1, averaging on from the next step.  The other post variables (ST,
 *   CL_AMP, CL1, TIME1, TIME2 and the sums) keep their values, zero at creation.
 * Every CALCCOEF while averaging runs calccoef.f90:156-190: CALC_VOR, the lift
 *   extremum test that sets ST and CL_AMP, the sums of U,V,P,T,VOR and of the
 *   coefficients, and the rms sums.
 * orc_post_final: POST_PROCESS with IPOST=1 (post_process.f90:19-36): averages
 *   into *out and the averaged fields into u,v,p,t,vor (any may be NULL); the
 *   reference overwrites its state with them at the end of the run, the oracle
 *   leaves the state alone.
 * orc_calc_vor: CALC_VOR (calc_vor.f90:14-58) into "VOR". */
void orc_post_begin(orc *o);
const orc_post *orc_post_record(const orc *o);
void orc_post_final(orc *o, orc_post *out, double *u, double *v, double *p, double *t, double *vor);
void orc_calc_vor(orc *o);

/* Raw access to any named array (NULL if unknown).  Names: "U","V","P","T",
 * "U_N","V_N","T_N","NLX","NLY","ADV","NLX_NM1","NLY_NM1","ADV_NM1","DIFX",
 * "DIFY","DIFT","S_U","S_V","UE","UW","VN","VS","X","Y","XG","YG","XIX","XIY",
 * "ETX","ETY","DJAC","Q11","Q12","Q22","DE","DW","DN","DS","THETA","AREA",
 * "AP","AE","AW","AN","AS","SU","DD","VOR","U_TA","V_TA","P_TA","T_TA","VOR_TA". */
double *orc_array(orc *o, const char *name);
int orc_size(const orc *o);         /* (NI+1)*(NJ+1) */
double orc_time(const orc *o);
void orc_set_time(orc *o, double t, int niter);
double orc_sum_area(const orc *o);

#ifdef __cplusplus
}
#endif
#endif
