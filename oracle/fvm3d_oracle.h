/*
 * fvm3d_oracle.h -- CPU restatement of the reference's 3-D LES time step
 * (LES/v2.3_LES-Reynolds stresses/, Fortran 90 + MPI), used ONLY as test
 * infrastructure: the 3-D parity tests call it as the checker.  The product never
 * links or calls this code.
 *
 * Pinned: in O3_FAITHFUL order it reproduces, to rounding (fields <= 1e-12
 * relative L2, coefficient records <= 1e-11), the golden fixtures made by
 * executing the reference's own Fortran sources of this solver
 * (tests/golden/make_golden.py, cases les3d_* and dns3d_*: LES and no-LES steps
 * on skewed and circular grids at the reference's Poisson settings).
 *
 * One process owns the whole domain.  The reference's halo exchange MPI_X
 * (mpi_x.f90) with a single periodic rank is a periodic copy: J=0 <- NJ-1,
 * J=NJ <- 1 (for every K), then K=0 <- NK-1, K=NK <- 1 (for every J).  Sums and
 * maxima over ranks (MPI_ALLREDUCE) become plain sums and maxima; quantities the
 * reference divides by the rank count NDIMK (the reference pressure of main.f90
 * and CPB of calccoef.f90) become plain averages over K.
 *
 * Arrays: Fortran order (0:NI, 0:NJ, 0:NK), element (i,j,k) at
 * i + (NI+1)*(j + (NJ+1)*k).  I radial (wall ghost 0, far ghost NI), J
 * circumferential and K spanwise, both periodic.  Node coordinates XG/YG/ZG use
 * the same storage for i=1..NI, j=1..NJ, k=1..NK.
 */
#ifndef FVM3D_ORACLE_H
#define FVM3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* O3_FAITHFUL: the reference's lexicographic line Gauss-Seidel sweeps with lagged
 *   periodic ghosts.  O3_GPU: red-black lines in every sweep (a line's colour is
 *   the parity of the sum of its two transverse indices), periodic neighbours read
 *   through index wrap, J and K lines of the predictor solved as cyclic systems. */
enum { O3_FAITHFUL = 0, O3_GPU = 1 };

typedef struct {
    int ni, nj, nk;        /* node counts; cells 1..NI-1 x 1..NJ-1 x 1..NK-1 */
    double re, pr, dt;
    double tin, t_wall;
    double resimax;        /* Poisson scaled-L1 tolerance */
    int nswpp;             /* Poisson sweep cap */
    int order;             /* O3_FAITHFUL or O3_GPU */
    int use_les;           /* dynamic Smagorinsky SGS terms (main.f90:59-69) */
    int les_zavg;          /* 0: coefficient averaged over the volume (the reference's);
                              1: Lilly least squares along K per (I,J), clipped at 0 */
    int thermal;           /* advance T (ITER_T, BCT) */
    int res_every;         /* O3_GPU: residual every k-th sweep */
    double ref_a;          /* reference area of the force coefficients (REF_A) */
} o3_params;

typedef struct {
    double time, cfl, cpb, cd, cl, cd_p, cd_v, cl_p, cl_v, nu;
    double cs2, ct2;       /* dynamic model coefficients of the step (volume mode) */
    int sweeps;
    double resid;
} o3_coeffs;

typedef struct o3 o3;

o3 *o3_create(const o3_params *p);
void o3_destroy(o3 *o);
/* GRID (grid.f90:46-320) and METRIC (metric.f90:33-520) from node coordinates. */
int o3_set_grid(o3 *o, const double *xg, const double *yg, const double *zg);
/* INIT (init.f90): uniform flow; du, dv, dw (may be NULL) added to the interior. */
int o3_init(o3 *o, const double *du, const double *dv, const double *dw);
/* Time steps (main.f90:33-147). */
int o3_step(o3 *o, int nsteps);
const o3_coeffs *o3_last_coeffs(const o3 *o);
/* Sub-steps for parity tests of single routines. */
void o3_sgs(o3 *o);                /* STRESS_TENSOR_DY */
void o3_test_filter(o3 *o, const double *in, double *out);
double *o3_array(o3 *o, const char *name);
/* Post-processing of the LES program (no effect on the flow).
 * o3_post_begin: POST_PROCESS with IPOST=0 (post_process.f90:8-59): the sums of
 *   U, V, W, P, T, their six products and the six SGS stresses -2 nu_t S_ij cleared,
 *   NITER_POS = 0; every later CALCCOEF adds the step (calccoef.f90:286-307).  The
 *   reference also switches DTIME to DTIME_POST there; the oracle keeps its dt.
 * o3_post_get: the averages of POST_PROCESS with IPOST=1 by name (see the .c). */
void o3_post_begin(o3 *o);
int o3_post_steps(const o3 *o);
int o3_post_get(o3 *o, const char *name, double *out);
int o3_size(const o3 *o);

#ifdef __cplusplus
}
#endif
#endif
