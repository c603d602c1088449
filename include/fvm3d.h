/*
 * fvm3d.h -- C-ABI of the GB300 3-D LES time step of the cylinder solver: the
 * reference's LES/v2.3_LES-Reynolds stresses/ driver (main.f90:33-147) on one GPU
 * owning the whole domain.  The reference's MPI halo exchange (mpi_x.f90) becomes
 * the periodic index wrap / ghost copy of a single rank.
 *
 * Arrays are the reference's (0:NI,0:NJ,0:NK) arrays in Fortran order, element
 * (i,j,k) at i + (NI+1)*(j + (NJ+1)*k): I radial, J circumferential (periodic
 * through the branch cut), K spanwise (periodic).  All entry points return an int
 * status (FVM_OK, FVM_ERR_*, as in fvm.h) and never abort.
 */
#ifndef FVM3D_H
#define FVM3D_H

#include "fvm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fvm3_params {
    int ni, nj, nk;        /* node counts (comdat_param.f90:6-8); NJ-1 and NK-1 must be even */
    double re, pr, dt;     /* RE, PR, DTIME (comdat_param.f90:37-45) */
    double tin, t_wall;    /* TIN, T_WALL */
    double resimax;        /* Poisson scaled-L1 tolerance (RESIMAX) */
    int nswpp;             /* Poisson sweep cap (NSWPP) */
    int use_les;           /* USE_LES: dynamic Smagorinsky SGS terms */
    int les_zavg;          /* 0: coefficient averaged over the volume (the reference's,
                              stress_tensor_dy.f90:486-517); 1: Lilly least squares along
                              the span per (I,J), clipped at zero */
    int thermal;           /* advance T (ITER_T, BCT) */
    int res_every;         /* Poisson residual every k-th sweep */
    double ref_a;          /* reference area of the force coefficients (REF_A) */
    int precision;         /* FVM_FP64, or FVM_MIXED: FP32 red-black Poisson sweeps on the
                              correction inside FP64 residual refinement; the SGS model, DIF,
                              NL, P_SOURCE, the AF right-hand sides and predictor line solves
                              in double-float (pairs of FP32, ~48-bit significands: the
                              Leonard term cancels to ~1e-6 of its operands, too far for
                              FP32); metrics, the Poisson residual, divergence, CALCCOEF and
                              the state FP64 */
    int refine_sweeps;     /* MIXED: FP32 sweeps per FP64 residual */
    int device;
    int tile_i_warps, tile_i_m;   /* tile of the I lines (Poisson and first AF sweep), 0 = automatic:
                                     warps per line group (1, 2, 4) and elements per thread
                                     (1..4; also 6, 8, 12 with one warp, 6, 8 with two);
                                     32 * warps * elements must cover NI-1 */
    int poisson_host_loop; /* 1 (default): the host replays the Poisson body until the
                              residual kernel reports completion (kernels visible to
                              profilers); 0: a graph while-node ends the loop on the device */
} fvm3_params;

typedef struct fvm3_coeffs {
    double time, cfl, cpb, cd, cl, cd_p, cd_v, cl_p, cl_v, nu;
    double cs2, ct2;       /* dynamic coefficients of the step (volume mode) */
    int sweeps;
    double resid;
} fvm3_coeffs;

struct fvm3_ctx;

/* Defaults: the reference's PARAMETERs where it has them (comdat_param.f90). */
int fvm3_default_params(fvm3_params *p);
int fvm3_create(const fvm3_params *p, struct fvm3_ctx **ctx);
int fvm3_destroy(struct fvm3_ctx *ctx);
const char *fvm3_last_error(const struct fvm3_ctx *ctx);
/* GRID + METRIC (grid.f90:46-320, metric.f90:33-520) from node coordinates and the
 * geometry part of INIT (init.f90:150-200). */
int fvm3_set_grid(struct fvm3_ctx *ctx, const double *xg, const double *yg, const double *zg);
/* INIT: uniform flow, du/dv/dw (may be NULL) added to the interior. */
int fvm3_init(struct fvm3_ctx *ctx, const double *du, const double *dv, const double *dw);
/* nsteps time steps (main.f90:33-147); out (may be NULL): the last step's record. */
int fvm3_step(struct fvm3_ctx *ctx, int nsteps, fvm3_coeffs *out);
/* Per-routine call points of the time loop, in the order fvm3_step runs them
 * (main.f90:33-147), for a driver that keeps some routines of its own:
 *   fvm3_begin_step     NITER_TIME, RTIME, U_N..T_N = U..T (main.f90:37-44), and the
 *                       far-field values BCU/BCT use during the step (bcu.f90:30-40)
 *   fvm3_contra_vel     CONTRA_VEL (contra_vel.f90:13-56)
 *   fvm3_nl             NLX..ADV kept as *_NM1, NL of U_N, V_N, W_N, T_N (main.f90:50-57)
 *   fvm3_stress_tensor  STRESS_TENSOR_DY and the SGS terms added to NLX..ADV
 *                       (main.f90:59-69); nothing when use_les = 0
 *   fvm3_dif            DIF of U_N, V_N, W_N, T_N (main.f90:72-75)
 *   fvm3_p_source       P_SOURCE(P) (p_source.f90:14-42)
 *   fvm3_iter_u         ITER_U of U (component 0), V (1) or W (2) (iter_u.f90:23-255)
 *   fvm3_remove_grad    u -= dt S/J, then BCU of U, V, W (main.f90:90-97)
 *   fvm3_iter_p         CONTRA_VEL, ITER_P, BCP (main.f90:99-104); resid and sweeps
 *                       may be NULL; FVM_ERR_NOCONV when the sweep cap ended it
 *   fvm3_correct        P_SOURCE, u += dt S/J, the far-field reference pressure,
 *                       BCU (main.f90:106-140)
 *   fvm3_iter_t         ITER_T, BCT (main.f90:143-145); nothing when thermal = 0
 *   fvm3_calccoef       CALCCOEF; out may be NULL */
int fvm3_begin_step(struct fvm3_ctx *ctx);
int fvm3_contra_vel(struct fvm3_ctx *ctx);
int fvm3_nl(struct fvm3_ctx *ctx);
int fvm3_stress_tensor(struct fvm3_ctx *ctx);
int fvm3_dif(struct fvm3_ctx *ctx);
int fvm3_p_source(struct fvm3_ctx *ctx);
int fvm3_iter_u(struct fvm3_ctx *ctx, int component);
int fvm3_remove_grad(struct fvm3_ctx *ctx);
int fvm3_iter_p(struct fvm3_ctx *ctx, double *resid, int *sweeps);
int fvm3_correct(struct fvm3_ctx *ctx);
int fvm3_iter_t(struct fvm3_ctx *ctx);
int fvm3_calccoef(struct fvm3_ctx *ctx, fvm3_coeffs *out);
/* TEST_FILTER(IN, OUT) (test_filter.f90:13-21): the [1,2,1]^3/64 box filter of the
 * host array in into the interior of the host array out (its other entries are
 * left as passed).  Needs the grid only. */
int fvm3_test_filter(struct fvm3_ctx *ctx, const double *in, double *out);
/* Post-processing of the LES program (post_process.f90, calccoef.f90:286-307):
 *   fvm3_post_begin  POST_PROCESS with IPOST=0: the sums cleared, NITER_POS = 0;
 *                    from the next step on every CALCCOEF (fvm3_step,
 *                    fvm3_calccoef) adds U, V, W, P, T, their six products and the
 *                    six SGS stresses -2 nu_t S_ij on the device.  The reference
 *                    also switches DTIME to DTIME_POST there; dt is left unchanged.
 *   fvm3_post_get    POST_PROCESS with IPOST=1, by name: "U_AVG","V_AVG","W_AVG",
 *                    "P_AVG","T_AVG"; the Reynolds stresses with their SGS part
 *                    "UU","UV","UW","VV","VW","WW"; the root mean squares
 *                    "U_RMS","V_RMS","W_RMS" (full arrays); the wall statistics
 *                    "CF_WALL","CP_WALL","NU_WALL" at out[j + (NJ+1) k] for the
 *                    wall cells (j, k), (NJ+1)*(NK+1) doubles.
 *   fvm3_post_steps  NITER_POS;  fvm3_post_end: averaging off. */
int fvm3_post_begin(struct fvm3_ctx *ctx);
int fvm3_post_get(struct fvm3_ctx *ctx, const char *name, double *out);
int fvm3_post_steps(struct fvm3_ctx *ctx, int *steps);
int fvm3_post_end(struct fvm3_ctx *ctx);
/* Named arrays ("U","V","W","P","T","NLX","NLY","NLZ","ADV","DJAC","SGS_X",...).
 * One array per call, synchronised before returning. */
int fvm3_get_array(struct fvm3_ctx *ctx, const char *name, double *out);
int fvm3_set_array(struct fvm3_ctx *ctx, const char *name, const double *in);
/* Host <-> device copies of the whole time-step state: the RESTART000.DAT contents
 * (RLES/writedata.f90:191-215, read back as RLES/init.f90:183-205) -- U, V, W, P, T
 * and the advection history NLX, NLY, NLZ, ADV, each (NI+1)*(NJ+1)*(NK+1) doubles in
 * the array layout above.  Any pointer may be NULL to skip that array.  One
 * asynchronous copy per array on the context's stream and a single synchronisation
 * per call; page-locked host buffers (cudaHostAlloc, cudaHostRegister) make each
 * copy one DMA transfer.  Upload requires fvm3_set_grid and stands in for
 * fvm3_init (a restart). */
int fvm3_upload_state(struct fvm3_ctx *ctx, const double *u, const double *v, const double *w, const double *p,
                      const double *t, const double *nlx, const double *nly, const double *nlz, const double *adv);
int fvm3_download_state(struct fvm3_ctx *ctx, double *u, double *v, double *w, double *p, double *t,
                        double *nlx, double *nly, double *nlz, double *adv);
/* One application of the SGS model (STRESS_TENSOR_DY) to the current state, for
 * tests of the model alone. */
int fvm3_sgs(struct fvm3_ctx *ctx, fvm3_coeffs *out);
/* Time of `sweeps` Poisson sweeps (both colours, state unchanged). */
int fvm3_time_sweeps(struct fvm3_ctx *ctx, int sweeps, double *ms_per_sweep);
int fvm3_get_stream(struct fvm3_ctx *ctx, void **stream);

#ifdef __cplusplus
}
#endif
#endif
