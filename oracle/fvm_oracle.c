/*
 * fvm_oracle.c -- CPU restatement of the reference's 2-D fractional 4-step
 * finite-volume cylinder solver (test infrastructure only; see fvm_oracle.h).
 *
 * Every routine below names the reference file:line it restates.  Reference
 * root: cylinder/cylinder_v3.0.3_AF_original 4step_face_nl/.  Floating-point
 * expressions keep the reference's left-to-right evaluation order and the
 * library is built with -ffp-contract=off so that results do not depend on the
 * host's fused multiply-add (x86 here, aarch64 on the GPU host).
 */
#include "fvm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct orc {
    orc_params p;
    int NI, NJ, NI1, n;
    double pi, pe, rtime;
    int niter_time;
    double sum_area;
    /* geometry */
    double *XG, *YG, *X, *Y, *XIX, *XIY, *ETX, *ETY, *DJAC, *Q11, *Q12, *Q22;
    double *DE, *DW, *DN, *DS, *THETA, *AREA, *PG;
    /* state */
    double *U, *V, *P, *T, *U_N, *V_N, *T_N;
    double *NLX, *NLY, *ADV, *NLX_NM1, *NLY_NM1, *ADV_NM1, *DIFX, *DIFY, *DIFT, *S_U, *S_V;
    /* fluxes and shared scratch (comdat_shared.f90:224-263) */
    double *U1, *U2, *UE, *UW, *VN, *VS, *AP, *AE, *AW, *AN, *AS, *SU, *DD;
    /* line work arrays */
    double *la, *lb, *lc, *ld, *lx, *lz, *lw, *lu, *lbb;
    /* wall controls (no reference counterpart): wall-normal blowing speed per J */
    double *BLOW;
    /* post-processing (comdat_shared.f90:149-160) */
    double *VOR, *U_TA, *V_TA, *P_TA, *T_TA, *VOR_TA;
    int ipost, toggle, niter_pos;
    double cl_nm1, cl1, st, cl_amp, time1, time2;
    double nu_ta, cd_ta, cl_ta, st_ta, cpb_ta, cl_amp_ta, rms_cd, rms_cl;
    orc_post post;
    orc_coeffs co;
};

#define ID(i, j) ((i) + o->NI1 * (j))

static double *zalloc(int n) { return (double *)calloc((size_t)n, sizeof(double)); }

orc *orc_create(const orc_params *p)
{
    if (!p || p->ni < 5 || p->nj < 5) return NULL;
    orc *o = (orc *)calloc(1, sizeof(orc));
    if (!o) return NULL;
    o->p = *p;
    if (o->p.res_every < 1) o->p.res_every = 1;
    o->NI = p->ni;
    o->NJ = p->nj;
    o->NI1 = p->ni + 1;
    o->n = (p->ni + 1) * (p->nj + 1);
    o->pi = 4.0 * atan(1.0); /* init.f90:15 */
    double **arrs[] = {&o->XG, &o->YG, &o->X, &o->Y, &o->XIX, &o->XIY, &o->ETX, &o->ETY,
                       &o->DJAC, &o->Q11, &o->Q12, &o->Q22, &o->DE, &o->DW, &o->DN, &o->DS,
                       &o->THETA, &o->AREA, &o->PG, &o->U, &o->V, &o->P, &o->T, &o->U_N,
                       &o->V_N, &o->T_N, &o->NLX, &o->NLY, &o->ADV, &o->NLX_NM1, &o->NLY_NM1,
                       &o->ADV_NM1, &o->DIFX, &o->DIFY, &o->DIFT, &o->S_U, &o->S_V, &o->U1,
                       &o->U2, &o->UE, &o->UW, &o->VN, &o->VS, &o->AP, &o->AE, &o->AW,
                       &o->AN, &o->AS, &o->SU, &o->DD, &o->VOR, &o->U_TA, &o->V_TA, &o->P_TA,
                       &o->T_TA, &o->VOR_TA};
    for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); k++) {
        *arrs[k] = zalloc(o->n);
        if (!*arrs[k]) { orc_destroy(o); return NULL; }
    }
    int m = (p->ni > p->nj ? p->ni : p->nj) + 2;
    o->la = zalloc(m); o->lb = zalloc(m); o->lc = zalloc(m);
    o->ld = zalloc(m); o->lx = zalloc(m); o->lz = zalloc(m);
    o->lw = zalloc(m); o->lu = zalloc(m); o->lbb = zalloc(m);
    o->BLOW = zalloc(p->nj + 1);
    if (!o->la || !o->lb || !o->lc || !o->ld || !o->lx || !o->lz || !o->lw || !o->lu || !o->lbb || !o->BLOW) {
        orc_destroy(o);
        return NULL;
    }
    return o;
}

void orc_destroy(orc *o)
{
    if (!o) return;
    double *arrs[] = {o->XG, o->YG, o->X, o->Y, o->XIX, o->XIY, o->ETX, o->ETY, o->DJAC,
                      o->Q11, o->Q12, o->Q22, o->DE, o->DW, o->DN, o->DS, o->THETA, o->AREA,
                      o->PG, o->U, o->V, o->P, o->T, o->U_N, o->V_N, o->T_N, o->NLX, o->NLY,
                      o->ADV, o->NLX_NM1, o->NLY_NM1, o->ADV_NM1, o->DIFX, o->DIFY, o->DIFT,
                      o->S_U, o->S_V, o->U1, o->U2, o->UE, o->UW, o->VN, o->VS, o->AP, o->AE,
                      o->AW, o->AN, o->AS, o->SU, o->DD, o->la, o->lb, o->lc, o->ld, o->lx, o->lz,
                      o->lw, o->lu, o->lbb, o->BLOW, o->VOR, o->U_TA, o->V_TA, o->P_TA, o->T_TA,
                      o->VOR_TA};
    for (size_t k = 0; k < sizeof(arrs) / sizeof(arrs[0]); k++) free(arrs[k]);
    free(o);
}

/* ------------------------------------------------------------------------- */
/* GRID: cell centres and ghost cells (grid.f90:56-114)                       */
/* ------------------------------------------------------------------------- */
static void grid_centres(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    double *X = o->X, *Y = o->Y, *XG = o->XG, *YG = o->YG;
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            X[ID(i, j)] = 0.25 * (((XG[ID(i + 1, j + 1)] + XG[ID(i + 1, j)]) + XG[ID(i, j + 1)]) + XG[ID(i, j)]);
            Y[ID(i, j)] = 0.25 * (((YG[ID(i + 1, j + 1)] + YG[ID(i + 1, j)]) + YG[ID(i, j + 1)]) + YG[ID(i, j)]);
        }
    for (int i = 1; i <= NI - 1; i++) { /* grid.f90:66-74 */
        X[ID(i, 0)] = X[ID(i, NJ - 1)]; Y[ID(i, 0)] = Y[ID(i, NJ - 1)];
        X[ID(i, NJ)] = X[ID(i, 1)];     Y[ID(i, NJ)] = Y[ID(i, 1)];
    }
    for (int j = 1; j <= NJ - 1; j++) { /* grid.f90:76-91: face midpoints, then mirrored */
        X[ID(0, j)] = (XG[ID(1, j + 1)] + XG[ID(1, j)]) * 0.5;
        Y[ID(0, j)] = (YG[ID(1, j + 1)] + YG[ID(1, j)]) * 0.5;
        X[ID(0, j)] = X[ID(0, j)] - (X[ID(1, j)] - X[ID(0, j)]);
        Y[ID(0, j)] = Y[ID(0, j)] - (Y[ID(1, j)] - Y[ID(0, j)]);
        X[ID(NI, j)] = (XG[ID(NI, j + 1)] + XG[ID(NI, j)]) * 0.5;
        Y[ID(NI, j)] = (YG[ID(NI, j + 1)] + YG[ID(NI, j)]) * 0.5;
        X[ID(NI, j)] = X[ID(NI, j)] + (X[ID(NI, j)] - X[ID(NI - 1, j)]);
        Y[ID(NI, j)] = Y[ID(NI, j)] + (Y[ID(NI, j)] - Y[ID(NI - 1, j)]);
    }
    /* grid.f90:94-113 corners */
    X[ID(0, 0)] = X[ID(0, NJ - 1)];   Y[ID(0, 0)] = Y[ID(0, NJ - 1)];
    X[ID(0, NJ)] = X[ID(0, 1)];       Y[ID(0, NJ)] = Y[ID(0, 1)];
    X[ID(NI, 0)] = X[ID(NI, NJ - 1)]; Y[ID(NI, 0)] = Y[ID(NI, NJ - 1)];
    X[ID(NI, NJ)] = X[ID(NI, 1)];     Y[ID(NI, NJ)] = Y[ID(NI, 1)];
}

static inline double fwd3(double a0, double a1, double a2) { return ((-(3.0 * a0)) + 4.0 * a1 - a2) / 2.0; }
static inline double bwd3(double a0, double a1, double a2) { return ((3.0 * a0 - 4.0 * a1) + a2) / 2.0; }

/* METRIC (metric.f90:18-168) */
static int metric(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    const double *X = o->X, *Y = o->Y;
    double *XXI = zalloc(o->n), *YXI = zalloc(o->n), *XET = zalloc(o->n), *YET = zalloc(o->n);
    if (!XXI || !YXI || !XET || !YET) { free(XXI); free(YXI); free(XET); free(YET); return -1; }
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) { /* metric.f90:21-27 */
            XXI[ID(i, j)] = (X[ID(i + 1, j)] - X[ID(i - 1, j)]) / 2.0;
            XET[ID(i, j)] = (X[ID(i, j + 1)] - X[ID(i, j - 1)]) / 2.0;
            YXI[ID(i, j)] = (Y[ID(i + 1, j)] - Y[ID(i - 1, j)]) / 2.0;
            YET[ID(i, j)] = (Y[ID(i, j + 1)] - Y[ID(i, j - 1)]) / 2.0;
        }
    for (int i = 1; i <= NI - 1; i++) { /* metric.f90:31-50 south/north rows, periodic */
        XXI[ID(i, 0)] = (X[ID(i + 1, 0)] - X[ID(i - 1, 0)]) / 2.0;
        XET[ID(i, 0)] = (X[ID(i, NJ)] - X[ID(i, NJ - 2)]) / 2.0;
        YXI[ID(i, 0)] = (Y[ID(i + 1, 0)] - Y[ID(i - 1, 0)]) / 2.0;
        YET[ID(i, 0)] = (Y[ID(i, NJ)] - Y[ID(i, NJ - 2)]) / 2.0;
        XXI[ID(i, NJ)] = (X[ID(i + 1, NJ)] - X[ID(i - 1, NJ)]) / 2.0;
        XET[ID(i, NJ)] = (X[ID(i, 2)] - X[ID(i, 0)]) / 2.0;
        YXI[ID(i, NJ)] = (Y[ID(i + 1, NJ)] - Y[ID(i - 1, NJ)]) / 2.0;
        YET[ID(i, NJ)] = (Y[ID(i, 2)] - Y[ID(i, 0)]) / 2.0;
    }
    for (int j = 1; j <= NJ - 1; j++) { /* metric.f90:52-70 west/east columns, one-sided */
        XXI[ID(0, j)] = fwd3(X[ID(0, j)], X[ID(1, j)], X[ID(2, j)]);
        XET[ID(0, j)] = (X[ID(0, j + 1)] - X[ID(0, j - 1)]) / 2.0;
        YXI[ID(0, j)] = fwd3(Y[ID(0, j)], Y[ID(1, j)], Y[ID(2, j)]);
        YET[ID(0, j)] = (Y[ID(0, j + 1)] - Y[ID(0, j - 1)]) / 2.0;
        XXI[ID(NI, j)] = bwd3(X[ID(NI, j)], X[ID(NI - 1, j)], X[ID(NI - 2, j)]);
        XET[ID(NI, j)] = (X[ID(NI, j + 1)] - X[ID(NI, j - 1)]) / 2.0;
        YXI[ID(NI, j)] = bwd3(Y[ID(NI, j)], Y[ID(NI - 1, j)], Y[ID(NI - 2, j)]);
        YET[ID(NI, j)] = (Y[ID(NI, j + 1)] - Y[ID(NI, j - 1)]) / 2.0;
    }
    /* metric.f90:71-110 corners */
    XXI[ID(0, 0)] = fwd3(X[ID(0, 0)], X[ID(1, 0)], X[ID(2, 0)]);
    XET[ID(0, 0)] = (X[ID(0, NJ)] - X[ID(0, NJ - 2)]) / 2.0;
    YXI[ID(0, 0)] = fwd3(Y[ID(0, 0)], Y[ID(1, 0)], Y[ID(2, 0)]);
    YET[ID(0, 0)] = (Y[ID(0, NJ)] - Y[ID(0, NJ - 2)]) / 2.0;
    XXI[ID(0, NJ)] = fwd3(X[ID(0, NJ)], X[ID(1, NJ)], X[ID(2, NJ)]);
    XET[ID(0, NJ)] = (X[ID(0, 2)] - X[ID(0, 0)]) / 2.0;
    YXI[ID(0, NJ)] = fwd3(Y[ID(0, NJ)], Y[ID(1, NJ)], Y[ID(2, NJ)]);
    YET[ID(0, NJ)] = (Y[ID(0, 2)] - Y[ID(0, 0)]) / 2.0;
    XXI[ID(NI, 0)] = bwd3(X[ID(NI, 0)], X[ID(NI - 1, 0)], X[ID(NI - 2, 0)]);
    XET[ID(NI, 0)] = (X[ID(NI, NJ)] - X[ID(NI, NJ - 2)]) / 2.0;
    YXI[ID(NI, 0)] = bwd3(Y[ID(NI, 0)], Y[ID(NI - 1, 0)], Y[ID(NI - 2, 0)]);
    YET[ID(NI, 0)] = (Y[ID(NI, NJ)] - Y[ID(NI, NJ - 2)]) / 2.0;
    XXI[ID(NI, NJ)] = bwd3(X[ID(NI, NJ)], X[ID(NI - 1, NJ)], X[ID(NI - 2, NJ)]);
    XET[ID(NI, NJ)] = (X[ID(NI, 2)] - X[ID(NI, 0)]) / 2.0;
    YXI[ID(NI, NJ)] = bwd3(Y[ID(NI, NJ)], Y[ID(NI - 1, NJ)], Y[ID(NI - 2, NJ)]);
    YET[ID(NI, NJ)] = (Y[ID(NI, 2)] - Y[ID(NI, 0)]) / 2.0;

    int bad = 0;
    for (int k = 0; k < o->n; k++) { /* metric.f90:114-156 */
        double dj = XXI[k] * YET[k] - YXI[k] * XET[k];
        o->DJAC[k] = dj;
        if (!(fabs(dj) >= 1.0e-15)) bad++; /* metric.f90:120 prints; here it is an error */
        o->XIX[k] = YET[k] / dj;
        o->XIY[k] = -(XET[k] / dj);
        o->ETX[k] = -(YXI[k] / dj);
        o->ETY[k] = XXI[k] / dj;
        o->Q11[k] = o->XIX[k] * o->XIX[k] + o->XIY[k] * o->XIY[k];
        o->Q12[k] = o->XIX[k] * o->ETX[k] + o->XIY[k] * o->ETY[k];
        o->Q22[k] = o->ETX[k] * o->ETX[k] + o->ETY[k] * o->ETY[k];
    }
    const double *J = o->DJAC;
    for (int j = 1; j <= NJ - 1; j++) /* metric.f90:159-168 */
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            o->DE[c] = 0.5 * (J[c] * o->Q11[c] + J[ID(i + 1, j)] * o->Q11[ID(i + 1, j)]);
            o->DW[c] = 0.5 * (J[c] * o->Q11[c] + J[ID(i - 1, j)] * o->Q11[ID(i - 1, j)]);
            o->DN[c] = 0.5 * (J[c] * o->Q22[c] + J[ID(i, j + 1)] * o->Q22[ID(i, j + 1)]);
            o->DS[c] = 0.5 * (J[c] * o->Q22[c] + J[ID(i, j - 1)] * o->Q22[ID(i, j - 1)]);
        }
    free(XXI); free(YXI); free(XET); free(YET);
    return bad ? -2 : 0;
}

int orc_set_grid(orc *o, const double *xg, const double *yg)
{
    if (!o || !xg || !yg) return -1;
    memcpy(o->XG, xg, sizeof(double) * (size_t)o->n);
    memcpy(o->YG, yg, sizeof(double) * (size_t)o->n);
    grid_centres(o);
    return metric(o);
}

/* ------------------------------------------------------------------------- */
/* Boundary conditions                                                        */
/* ------------------------------------------------------------------------- */
enum { BC_U = 0, BC_V = 1, BC_T = 2 };

/* BCU / BCV / BCT (bcu.f90:10-51, bcv.f90, bct.f90).  The reference loops the
 * wall and far-field rows over J=0..NJ; the J=0 and J=NJ entries it writes are
 * overwritten by the branch-cut copy and its scratch rows J=0/NJ are never
 * read, so only J=1..NJ-1 are restated (the reference's far-field formula at
 * J=0/NJ reads outside the array). */
static void bc_field(orc *o, int kind, double *phi, const double *phin)
{
    const int NI = o->NI, NJ = o->NJ;
    const double pi = o->pi;
    for (int j = 1; j <= NJ - 1; j++) {
        double th = o->THETA[ID(0, j)];
        double f;
        if (kind == BC_U) f = o->p.vel_rot * (-sin(th)) + o->BLOW[j] * cos(th);
        else if (kind == BC_V) f = o->p.vel_rot * cos(th) + o->BLOW[j] * sin(th);
        else f = o->p.t_wall;
        int c1 = ID(1, j);
        o->AP[c1] = o->AP[c1] + o->AW[c1];
        o->SU[c1] = o->SU[c1] + (2.0 * o->AW[c1]) * f;
        o->AW[c1] = 0.0;
        phi[ID(0, j)] = (-phi[c1]) + 2.0 * f;
    }
    for (int j = 1; j <= NJ - 1; j++) {
        double th = o->THETA[ID(NI, j)];
        double f;
        if (th >= 0.5 * pi && th <= 1.5 * pi) {
            f = (kind == BC_U) ? o->p.uin : (kind == BC_V) ? o->p.vin : o->p.tin;
        } else { /* convective outflow from the step-n field (bcu.f90:30-32) */
            const double *q = phin;
            double a = 0.5 * (o->XIX[ID(NI, j)] + o->XIX[ID(NI - 1, j)]);
            double b = (0.5 * (o->ETX[ID(NI, j)] + o->ETX[ID(NI - 1, j)])) * 0.25;
            double dq = ((q[ID(NI, j + 1)] + q[ID(NI - 1, j + 1)]) - q[ID(NI, j - 1)]) - q[ID(NI - 1, j - 1)];
            f = 0.5 * (q[ID(NI, j)] + q[ID(NI - 1, j)])
                - (o->p.dt * o->p.uin) * (a * (q[ID(NI, j)] - q[ID(NI - 1, j)]) + b * dq);
        }
        int cm = ID(NI - 1, j);
        o->AP[cm] = o->AP[cm] + o->AE[cm];
        o->SU[cm] = o->SU[cm] + (2.0 * o->AE[cm]) * f;
        o->AE[cm] = 0.0;
        phi[ID(NI, j)] = (-phi[cm]) + 2.0 * f;
    }
    for (int i = 0; i <= NI; i++) { /* branch cut */
        phi[ID(i, 0)] = phi[ID(i, NJ - 1)];
        phi[ID(i, NJ)] = phi[ID(i, 1)];
    }
}

static void bcu(orc *o) { bc_field(o, BC_U, o->U, o->U_N); }
static void bcv(orc *o) { bc_field(o, BC_V, o->V, o->V_N); }
static void bct(orc *o) { bc_field(o, BC_T, o->T, o->T_N); }

/* BCP (bcp.f90:8-42) */
static void bcp(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    double *P = o->P;
    for (int j = 1; j <= NJ - 1; j++) {
        int c1 = ID(1, j);
        o->AP[c1] = o->AP[c1] - o->AW[c1];
        o->AW[c1] = 0.0;
        P[ID(0, j)] = P[c1];
        o->AE[ID(NI - 1, j)] = 0.0;
        P[ID(NI, j)] = (3.0 * P[ID(NI - 1, j)] - 3.0 * P[ID(NI - 2, j)]) + P[ID(NI - 3, j)];
    }
    for (int i = 0; i <= NI; i++) {
        P[ID(i, 0)] = P[ID(i, NJ - 1)];
        P[ID(i, NJ)] = P[ID(i, 1)];
    }
}

/* ------------------------------------------------------------------------- */
/* INIT (init.f90:17-137)                                                     */
/* ------------------------------------------------------------------------- */
static double theta_of(double x, double y, double pi)
{   /* init.f90:94-100: quadrant fix-up of DATAN(Y/X) via the sign of DASIN(Y/R) */
    double r = sqrt(x * x + y * y);
    double th = atan(y / x);
    double s = asin(y / r);
    if (th >= 0.0 && s > 0.0) th = th;
    else if (th < 0.0 && s > 0.0) th = pi + th;
    else if (th >= 0.0 && s <= 0.0) th = pi + th;
    else if (th < 0.0 && s < 0.0) th = 2.0 * pi + th;
    return th;
}

int orc_init(orc *o, const double *du, const double *dv)
{
    if (!o) return -1;
    const int NI = o->NI, NJ = o->NJ;
    o->niter_time = 0;
    o->rtime = 0.0;
    for (int k = 0; k < o->n; k++) {
        o->U[k] = 1.0; o->U_N[k] = 1.0;
        o->V[k] = 0.0; o->V_N[k] = 0.0;
        o->T[k] = 0.0; o->T_N[k] = 0.0;
        o->P[k] = 0.0;
        o->NLX[k] = 0.0; o->NLY[k] = 0.0; o->ADV[k] = 0.0;
        o->THETA[k] = 0.0; /* THETA is computed below, after the boundary calls */
        o->AP[k] = o->AE[k] = o->AW[k] = o->AN[k] = o->AS[k] = o->SU[k] = 0.0;
    }
    /* seeded perturbation of the uniform start (no reference counterpart) */
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            if (du) o->U[ID(i, j)] += du[ID(i, j)];
            if (dv) o->V[ID(i, j)] += dv[ID(i, j)];
        }
    bcu(o); bcv(o); bcp(o); bct(o); /* init.f90:33-36, with THETA still zero */
    memcpy(o->U_N, o->U, sizeof(double) * (size_t)o->n);
    memcpy(o->V_N, o->V, sizeof(double) * (size_t)o->n);
    memcpy(o->T_N, o->T, sizeof(double) * (size_t)o->n);
    for (int k = 0; k < o->n; k++) o->THETA[k] = theta_of(o->X[k], o->Y[k], o->pi);
    o->sum_area = 0.0; /* init.f90:120-128 */
    for (int j = 1; j <= NJ - 1; j++) {
        double dx = o->XG[ID(1, j + 1)] - o->XG[ID(1, j)];
        double dy = o->YG[ID(1, j + 1)] - o->YG[ID(1, j)];
        o->AREA[ID(1, j)] = sqrt(dx * dx + dy * dy);
        o->sum_area = o->sum_area + o->AREA[ID(1, j)];
    }
    o->pe = o->p.re * o->p.pr; /* init.f90:130 */
    memset(&o->co, 0, sizeof(o->co));
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Wall controls (no reference counterpart)                                   */
/* ------------------------------------------------------------------------- */
/* Wall rotation rate omega (the reference's VEL_ROT, bcu.f90:13) and a
 * wall-normal blowing speed b_J per wall cell J=1..NJ-1: the wall velocity of
 * cell J becomes omega*(-sin th, cos th) + b_J*(cos th, sin th), th = THETA(0,J),
 * and the wall face flux UW(1,J), zero in the reference (contra_vel.f90:125), is
 * b_J times the face value of J*(xi_x cos th + xi_y sin th) averaged over the
 * ghost and first cells.  With b = 0 the step is the reference's. */
void orc_set_controls(orc *o, double omega, const double *blow)
{
    o->p.vel_rot = omega;
    for (int j = 0; j <= o->NJ; j++) o->BLOW[j] = 0.0;
    if (blow)
        for (int j = 1; j <= o->NJ - 1; j++) o->BLOW[j] = blow[j - 1];
}

static double wall_flux(const orc *o, int j)
{
    const double th = o->THETA[ID(0, j)], ct = cos(th), st = sin(th);
    const int c0 = ID(0, j), c1 = ID(1, j);
    return 0.5 * (o->DJAC[c0] * (o->XIX[c0] * ct + o->XIY[c0] * st) + o->DJAC[c1] * (o->XIX[c1] * ct + o->XIY[c1] * st));
}

/* ------------------------------------------------------------------------- */
/* Explicit operators                                                         */
/* ------------------------------------------------------------------------- */
/* CONTRA_VEL, FLAG=0 (contra_vel.f90:9-21,125) */
void orc_contra_vel(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    for (int k = 0; k < o->n; k++) {
        o->U1[k] = o->XIX[k] * o->U[k] + o->XIY[k] * o->V[k];
        o->U2[k] = o->ETX[k] * o->U[k] + o->ETY[k] * o->V[k];
    }
    const double *J = o->DJAC, *U1 = o->U1, *U2 = o->U2;
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            o->UE[c] = 0.5 * (J[c] * U1[c] + J[ID(i + 1, j)] * U1[ID(i + 1, j)]);
            o->UW[c] = 0.5 * (J[c] * U1[c] + J[ID(i - 1, j)] * U1[ID(i - 1, j)]);
            o->VN[c] = 0.5 * (J[c] * U2[c] + J[ID(i, j + 1)] * U2[ID(i, j + 1)]);
            o->VS[c] = 0.5 * (J[c] * U2[c] + J[ID(i, j - 1)] * U2[ID(i, j - 1)]);
        }
    for (int j = 1; j <= NJ - 1; j++) o->UW[ID(1, j)] = wall_flux(o, j) * o->BLOW[j];
}

/* NL (nl.f90:21-27): face-flux advection */
static void nl(orc *o, const double *in, double *out)
{
    const int NI = o->NI, NJ = o->NJ;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            double t1 = (o->UE[c] * 0.5) * (in[c] + in[ID(i + 1, j)]);
            double t2 = (o->UW[c] * 0.5) * (in[c] + in[ID(i - 1, j)]);
            double t3 = (o->VN[c] * 0.5) * (in[c] + in[ID(i, j + 1)]);
            double t4 = (o->VS[c] * 0.5) * (in[c] + in[ID(i, j - 1)]);
            out[c] = 1.0 * (((t1 - t2) + t3) - t4);
        }
}

/* DIF_DIAGONAL (dif_diagonal.f90:13-23): cross-derivative term with J*Q12 */
static void dif_diagonal(orc *o, const double *f, double *out)
{
    const int NI = o->NI, NJ = o->NJ;
    const double *J = o->DJAC, *Q = o->Q12;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int e = ID(i + 1, j), w = ID(i - 1, j), nn = ID(i, j + 1), s = ID(i, j - 1);
            double t1 = (J[e] * Q[e]) * (f[ID(i + 1, j + 1)] - f[ID(i + 1, j - 1)]);
            double t2 = (J[w] * Q[w]) * (f[ID(i - 1, j + 1)] - f[ID(i - 1, j - 1)]);
            double t3 = (J[nn] * Q[nn]) * (f[ID(i + 1, j + 1)] - f[ID(i - 1, j + 1)]);
            double t4 = (J[s] * Q[s]) * (f[ID(i + 1, j - 1)] - f[ID(i - 1, j - 1)]);
            out[ID(i, j)] = 0.25 * (((t1 - t2) + t3) - t4);
        }
}

/* Cell whose cross term DIF and ITER_P add to cell (i,j).  Both routines add the
 * whole array DD(0:NI,0:NJ) to an expression over the interior section
 * (1:NI-1,1:NJ-1) (dif.f90:15-23, iter_p.f90:27-30).  The shapes do not conform;
 * compiled code evaluates the sum element by element by position, so interior
 * cell (i,j) receives DD(i-1,j-1) -- zero on row 0 and column 0, which no routine
 * writes.  dd_positional=0 selects the cell's own term instead. */
static inline int dd_at(const orc *o, int i, int j)
{
    return o->p.dd_positional ? ID(i - 1, j - 1) : ID(i, j);
}

/* DIF (dif.f90:13-23) */
static void dif(orc *o, const double *in, double *out)
{
    const int NI = o->NI, NJ = o->NJ;
    dif_diagonal(o, in, o->DD);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            double a = o->DE[c] * (in[ID(i + 1, j)] - in[c]);
            double b = o->DW[c] * (in[ID(i - 1, j)] - in[c]);
            double d = o->DN[c] * (in[ID(i, j + 1)] - in[c]);
            double e = o->DS[c] * (in[ID(i, j - 1)] - in[c]);
            out[c] = 1.0 * ((((a + b) + d) + e) + o->DD[dd_at(o, i, j)]);
        }
}

/* P_SOURCE (p_source.f90:9-27): -J grad p by face differences */
static void p_source(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    const double *J = o->DJAC, *P = o->P;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int e = ID(i + 1, j), w = ID(i - 1, j), nn = ID(i, j + 1), s = ID(i, j - 1);
            double a = ((((J[e] * o->XIX[e]) * P[e] - (J[w] * o->XIX[w]) * P[w]) + (J[nn] * o->ETX[nn]) * P[nn]) - (J[s] * o->ETX[s]) * P[s]);
            double b = ((((J[e] * o->XIY[e]) * P[e] - (J[w] * o->XIY[w]) * P[w]) + (J[nn] * o->ETY[nn]) * P[nn]) - (J[s] * o->ETY[s]) * P[s]);
            o->S_U[ID(i, j)] = -(0.5 * a);
            o->S_V[ID(i, j)] = -(0.5 * b);
        }
}

/* ------------------------------------------------------------------------- */
/* Line solvers                                                               */
/* ------------------------------------------------------------------------- */
static inline int jwrap(const orc *o, int j)
{
    if (j == 0) return o->NJ - 1;
    if (j == o->NJ) return 1;
    return j;
}

/* One radial line j: Thomas along i with the reference's recurrences
 * (iter_u.f90:52-64, lisolv.f90:72-84).  B(0)=0 is the reference's never-written
 * SAVE element.  jn/js are the rows read for the explicit neighbour terms. */
static void radial_line(orc *o, double *phi, int j, int jn, int js, double *B, double *D)
{
    const int NI = o->NI;
    B[0] = 0.0;
    for (int i = 1; i <= NI - 1; i++) {
        int c = ID(i, j);
        double A = -o->AW[c];
        D[i] = o->AP[c] - A * B[i - 1];
        B[i] = -o->AE[c] / D[i];
        double C = (o->AN[c] * phi[ID(i, jn)] + o->AS[c] * phi[ID(i, js)]) + o->SU[c];
        phi[c] = (C - A * phi[ID(i - 1, j)]) / D[i];
    }
    for (int i = NI - 1; i >= 1; i--) phi[ID(i, j)] = phi[ID(i, j)] - B[i] * phi[ID(i + 1, j)];
}

/* Radial-line sweep: faithful order j = 1..NJ-1 reading the stored rows j+-1
 * (ghost rows at the branch cut), or zebra order with periodic wrap. */
static void sweep_radial(orc *o, double *phi)
{
    const int NI = o->NI, NJ = o->NJ;
    if (o->p.order == ORC_FAITHFUL) {
        for (int j = 1; j <= NJ - 1; j++) radial_line(o, phi, j, j + 1, j - 1, o->lb, o->ld);
    } else {
        /* the lines of one colour are independent: any thread count gives the
           same bits (each thread has its own recurrence scratch) */
        for (int c = 1; c >= 0; c--) { /* odd lines (colour 0) first, then even lines */
#pragma omp parallel
            {
                double B[NI + 1], D[NI + 1];
#pragma omp for schedule(static)
                for (int j = 2 - c; j <= NJ - 1; j += 2)
                    radial_line(o, phi, j, jwrap(o, j + 1), jwrap(o, j - 1), B, D);
            }
        }
    }
}

/* Tridiagonal solve a_k x_{k-1} + b_k x_k + c_k x_{k+1} = d_k, k=1..n (a_1, c_n unused). */
static void thomas(int n, const double *a, const double *b, const double *c, const double *d, double *x, double *w)
{
    double bet = b[1];
    x[1] = d[1] / bet;
    for (int k = 2; k <= n; k++) {
        w[k] = c[k - 1] / bet;
        bet = b[k] - a[k] * w[k];
        x[k] = (d[k] - a[k] * x[k - 1]) / bet;
    }
    for (int k = n - 1; k >= 1; k--) x[k] -= w[k + 1] * x[k + 1];
}

/* Cyclic tridiagonal solve by Sherman-Morrison: row 1 couples x_n through a_1,
 * row n couples x_1 through c_n.  bb, u, z, w are work arrays of length n+1. */
static void cyclic(int n, const double *a, const double *b, const double *c, const double *d, double *x,
                   double *bb, double *u, double *z, double *w)
{
    double gamma = -b[1];
    for (int k = 1; k <= n; k++) { bb[k] = b[k]; u[k] = 0.0; }
    bb[1] = b[1] - gamma;
    bb[n] = b[n] - a[1] * c[n] / gamma;
    thomas(n, a, bb, c, d, x, w);
    u[1] = gamma;
    u[n] = c[n];
    thomas(n, a, bb, c, u, z, w);
    double fact = (x[1] + a[1] * x[n] / gamma) / (1.0 + z[1] + a[1] * z[n] / gamma);
    for (int k = 1; k <= n; k++) x[k] -= fact * z[k];
}

/* Circumferential-line sweep of the predictor (second AF sweep).
 * Faithful: i = 1..NI-1 in order, Thomas along j with the lagged ghost values
 * phi(i,0), phi(i,NJ) (iter_u.f90:104-119).
 * GPU: zebra over i (odd lines first), each line a cyclic tridiagonal system. */
static void sweep_theta(orc *o, double *phi)
{
    const int NI = o->NI, NJ = o->NJ;
    if (o->p.order == ORC_FAITHFUL) {
        double *B = o->lb, *D = o->ld;
        B[0] = 0.0;
        for (int i = 1; i <= NI - 1; i++) {
            for (int j = 1; j <= NJ - 1; j++) {
                int c = ID(i, j);
                double A = -o->AS[c];
                D[j] = o->AP[c] - A * B[j - 1];
                B[j] = -o->AN[c] / D[j];
                double C = (o->AE[c] * phi[ID(i + 1, j)] + o->AW[c] * phi[ID(i - 1, j)]) + o->SU[c];
                phi[c] = (C - A * phi[ID(i, j - 1)]) / D[j];
            }
            for (int j = NJ - 1; j >= 1; j--) phi[ID(i, j)] = phi[ID(i, j)] - B[j] * phi[ID(i, j + 1)];
        }
        return;
    }
    const int n = NJ - 1;
    for (int col = 1; col >= 0; col--) {
#pragma omp parallel
        {
            double a[n + 2], b[n + 2], cc[n + 2], d[n + 2], x[n + 2], bb[n + 2], u[n + 2], z[n + 2], w[n + 2];
#pragma omp for schedule(static)
            for (int i = 2 - col; i <= NI - 1; i += 2) {
                for (int j = 1; j <= n; j++) {
                    int c = ID(i, j);
                    a[j] = -o->AS[c];
                    b[j] = o->AP[c];
                    cc[j] = -o->AN[c];
                    d[j] = (o->AE[c] * phi[ID(i + 1, j)] + o->AW[c] * phi[ID(i - 1, j)]) + o->SU[c];
                }
                cyclic(n, a, b, cc, d, x, bb, u, z, w);
                for (int j = 1; j <= n; j++) phi[ID(i, j)] = x[j];
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Approximate-factorisation predictor (iter_u.f90, iter_v.f90, iter_T.f90)    */
/* ------------------------------------------------------------------------- */
/* Face-averaged J*m1^2 coefficient pair and the cross term of one AF factor. */
static void af_coeffs(orc *o, const double *m1, const double *m2, double rek)
{
    const int NI = o->NI, NJ = o->NJ;
    const double *J = o->DJAC;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j), e = ID(i + 1, j), w = ID(i - 1, j), nn = ID(i, j + 1), s = ID(i, j - 1);
            o->AE[c] = 0.5 * (J[c] * (m1[c] * m1[c]) + J[e] * (m1[e] * m1[e]));
            o->AW[c] = 0.5 * (J[c] * (m1[c] * m1[c]) + J[w] * (m1[w] * m1[w]));
            o->AN[c] = 0.5 * (J[c] * (m2[c] * m2[c]) + J[nn] * (m2[nn] * m2[nn]));
            o->AS[c] = 0.5 * (J[c] * (m2[c] * m2[c]) + J[s] * (m2[s] * m2[s]));
            o->AP[c] = (((((2.0 * rek) * J[c]) / o->p.dt + o->AE[c]) + o->AW[c]) + o->AN[c]) + o->AS[c];
        }
}

static void af_cross(orc *o, const double *m1, const double *m2, const double *f)
{
    const int NI = o->NI, NJ = o->NJ;
    const double *J = o->DJAC;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int e = ID(i + 1, j), w = ID(i - 1, j), nn = ID(i, j + 1), s = ID(i, j - 1);
            double t1 = ((J[e] * m1[e]) * m2[e]) * (f[ID(i + 1, j + 1)] - f[ID(i + 1, j - 1)]);
            double t2 = ((J[w] * m1[w]) * m2[w]) * (f[ID(i - 1, j + 1)] - f[ID(i - 1, j - 1)]);
            double t3 = ((J[nn] * m1[nn]) * m2[nn]) * (f[ID(i + 1, j + 1)] - f[ID(i - 1, j + 1)]);
            double t4 = ((J[s] * m1[s]) * m2[s]) * (f[ID(i + 1, j - 1)] - f[ID(i - 1, j - 1)]);
            o->DD[ID(i, j)] = 0.25 * (((t1 - t2) + t3) - t4);
        }
}

static void iter_af(orc *o, int kind, double *phi, const double *phin, const double *nlx,
                    const double *nlm1, const double *difx, const double *src)
{
    const int NI = o->NI, NJ = o->NJ;
    const double rek = (kind == BC_T) ? o->pe : o->p.re;
    /* first factor: x-split coefficients (iter_u.f90:13-46) */
    af_coeffs(o, o->XIX, o->ETX, rek);
    af_cross(o, o->XIX, o->ETX, phi);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            double s = ((((2.0 * rek) * o->DJAC[c]) / o->p.dt) * phin[c] - (3.0 * rek) * nlx[c]) + (1.0 * rek) * nlm1[c];
            s = s + difx[c];
            if (src) s = s + (2.0 * rek) * src[c];
            o->SU[c] = s + o->DD[c];
        }
    bc_field(o, kind, phi, phin);
    sweep_radial(o, phi);
    /* second factor: y-split coefficients (iter_u.f90:68-101) */
    af_coeffs(o, o->XIY, o->ETY, rek);
    /* ITER_T builds this cross term from V (iter_T.f90:89-95) */
    const double *fx = (kind == BC_T && o->p.iter_t_bug) ? o->V : phi;
    af_cross(o, o->XIY, o->ETY, fx);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            o->SU[c] = (((2.0 * rek) * o->DJAC[c]) / o->p.dt) * phi[c] + o->DD[c];
        }
    bc_field(o, kind, phi, phin);
    sweep_theta(o, phi);
}

void orc_iter_u(orc *o) { iter_af(o, BC_U, o->U, o->U_N, o->NLX, o->NLX_NM1, o->DIFX, o->S_U); }
void orc_iter_v(orc *o) { iter_af(o, BC_V, o->V, o->V_N, o->NLY, o->NLY_NM1, o->DIFY, o->S_V); }

/* ------------------------------------------------------------------------- */
/* Pressure Poisson (iter_p.f90:12-51, lisolv.f90:18-33)                       */
/* ------------------------------------------------------------------------- */
static double residual(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    const double *P = o->P;
    double resip = 0.0, dum = 0.0;
    for (int j = 1; j <= NJ - 1; j++) {
        int jn = j + 1, js = j - 1;
        if (o->p.order != ORC_FAITHFUL) { jn = jwrap(o, jn); js = jwrap(o, js); }
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            double r = ((((o->AE[c] * P[ID(i + 1, j)] + o->AW[c] * P[ID(i - 1, j)]) + o->AN[c] * P[ID(i, jn)])
                         + o->AS[c] * P[ID(i, js)]) + o->SU[c]) - o->AP[c] * P[c];
            resip = resip + fabs(r);
            dum = dum + fabs(o->AP[c] * P[c]);
        }
    }
    return resip / dum;
}

static int iter_p(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    for (int k = 0; k < o->n; k++) {
        o->AP[k] = (((-o->DE[k]) - o->DW[k]) - o->DN[k]) - o->DS[k];
        o->AE[k] = -o->DE[k];
        o->AW[k] = -o->DW[k];
        o->AN[k] = -o->DN[k];
        o->AS[k] = -o->DS[k];
        o->SU[k] = 0.0;
    }
    const double rdt = 1.0 / o->p.dt;
    int niter = 0;
    double resip = 0.0;
    for (;;) {
        niter = niter + 1;
        dif_diagonal(o, o->P, o->DD);
#pragma omp parallel for schedule(static)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                int c = ID(i, j);
                o->SU[c] = rdt * (((o->UE[c] - o->UW[c]) + o->VN[c]) - o->VS[c]) - o->DD[dd_at(o, i, j)];
            }
        bcp(o);
        sweep_radial(o, o->P);
        int check = (o->p.order == ORC_FAITHFUL) || (niter % o->p.res_every == 0) || (niter >= o->p.nswpp);
        if (check) {
            resip = residual(o);
            if (!(resip > o->p.resimax && niter < o->p.nswpp)) break;
        }
    }
    o->co.sweeps = niter;
    o->co.resid = resip;
    return niter;
}

/* ------------------------------------------------------------------------- */
/* Time step (Main.f90:48-114)                                                */
/* ------------------------------------------------------------------------- */
void orc_begin_step(orc *o)
{
    o->niter_time = o->niter_time + 1;
    o->rtime = o->rtime + o->p.dt;
    memcpy(o->U_N, o->U, sizeof(double) * (size_t)o->n);
    memcpy(o->V_N, o->V, sizeof(double) * (size_t)o->n);
    memcpy(o->T_N, o->T, sizeof(double) * (size_t)o->n);
}

void orc_explicit(orc *o)
{
    memcpy(o->NLX_NM1, o->NLX, sizeof(double) * (size_t)o->n);
    memcpy(o->NLY_NM1, o->NLY, sizeof(double) * (size_t)o->n);
    memcpy(o->ADV_NM1, o->ADV, sizeof(double) * (size_t)o->n);
    nl(o, o->U_N, o->NLX);
    nl(o, o->V_N, o->NLY);
    nl(o, o->T_N, o->ADV);
    dif(o, o->U_N, o->DIFX);
    dif(o, o->V_N, o->DIFY);
    dif(o, o->T_N, o->DIFT);
    p_source(o);
}

static void grad_update(orc *o, double sign)
{
    const int NI = o->NI, NJ = o->NJ;
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            int c = ID(i, j);
            double du = (o->S_U[c] * o->p.dt) / o->DJAC[c];
            double dv = (o->S_V[c] * o->p.dt) / o->DJAC[c];
            if (sign < 0) { o->U[c] = o->U[c] - du; o->V[c] = o->V[c] - dv; }
            else { o->U[c] = o->U[c] + du; o->V[c] = o->V[c] + dv; }
        }
}

void orc_remove_grad(orc *o)
{
    grad_update(o, -1.0); /* Main.f90:80-84 */
    bcu(o);
    bcv(o);
}

int orc_iter_p(orc *o)
{
    orc_contra_vel(o); /* Main.f90:91 */
    int s = iter_p(o);
    bcp(o);
    return s;
}

void orc_correct(orc *o)
{
    p_source(o); /* Main.f90:97-107 */
    grad_update(o, +1.0);
    bcu(o);
    bcv(o);
}

void orc_iter_t(orc *o)
{
    iter_af(o, BC_T, o->T, o->T_N, o->ADV, o->ADV_NM1, o->DIFT, NULL);
    bct(o);
}

/* CALC_VOR (calc_vor.f90:14-58): cell-centre vorticity, one-sided (extrapolated
 * ghost) differences on the I=0 and I=NI rows, branch-cut rows copied. */
void orc_calc_vor(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    const double *U = o->U, *V = o->V;
    double *W = o->VOR;
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            const int c = ID(i, j);
            W[c] = (((o->XIX[c] * 0.5) * (V[ID(i + 1, j)] - V[ID(i - 1, j)]) +
                     (o->ETX[c] * 0.5) * (V[ID(i, j + 1)] - V[ID(i, j - 1)])) -
                    (o->XIY[c] * 0.5) * (U[ID(i + 1, j)] - U[ID(i - 1, j)])) -
                   (o->ETY[c] * 0.5) * (U[ID(i, j + 1)] - U[ID(i, j - 1)]);
        }
    for (int j = 1; j <= NJ - 1; j++) {
        int i = 0, c = ID(i, j);
        W[c] = (((o->XIX[c] * 0.5) * (V[ID(i + 1, j)] - ((3.0 * V[c] - 3.0 * V[ID(i + 1, j)]) + V[ID(i + 2, j)])) +
                 (o->ETX[c] * 0.5) * (V[ID(i, j + 1)] - V[ID(i, j - 1)])) -
                (o->XIY[c] * 0.5) * (U[ID(i + 1, j)] - ((3.0 * U[c] - 3.0 * U[ID(i + 1, j)]) + U[ID(i + 2, j)]))) -
               (o->ETY[c] * 0.5) * (U[ID(i, j + 1)] - U[ID(i, j - 1)]);
        i = NI;
        c = ID(i, j);
        W[c] = (((o->XIX[c] * 0.5) * (((3.0 * V[c] - 3.0 * V[ID(i - 1, j)]) + V[ID(i - 2, j)]) - V[ID(i - 1, j)]) +
                 (o->ETX[c] * 0.5) * (V[ID(i, j + 1)] - V[ID(i, j - 1)])) -
                (o->XIY[c] * 0.5) * (((3.0 * U[c] - 3.0 * U[ID(i - 1, j)]) + U[ID(i - 2, j)]) - U[ID(i - 1, j)])) -
               (o->ETY[c] * 0.5) * (U[ID(i, j + 1)] - U[ID(i, j - 1)]);
    }
    for (int i = 0; i <= NI; i++) {
        W[ID(i, 0)] = W[ID(i, NJ - 1)];
        W[ID(i, NJ)] = W[ID(i, 1)];
    }
}

/* POST_PROCESS, IPOST=0 branch (post_process.f90:8-16). */
void orc_post_begin(orc *o)
{
    o->niter_pos = 0;
    o->toggle = 1;
    o->ipost = 1;
}

/* The post-processing block of CALCCOEF (calccoef.f90:156-190). */
static void post_step(orc *o)
{
    orc_calc_vor(o);
    o->niter_pos = o->niter_pos + 1;
    const double cl = o->co.cl, rtime = o->rtime;
    if ((double)o->toggle * (cl - o->cl_nm1) < 0.0) { /* lift extremum: half period */
        o->toggle = -1 * o->toggle;
        o->st = 1.0 / (rtime - o->time2);
        o->time2 = o->time1;
        o->time1 = rtime;
        o->cl_amp = fabs(cl - o->cl1) / 2.0;
        o->cl1 = cl;
    }
    for (int c = 0; c < o->n; c++) {
        o->U_TA[c] = o->U_TA[c] + o->U[c];
        o->V_TA[c] = o->V_TA[c] + o->V[c];
        o->P_TA[c] = o->P_TA[c] + o->P[c];
        o->T_TA[c] = o->T_TA[c] + o->T[c];
        o->VOR_TA[c] = o->VOR_TA[c] + o->VOR[c];
    }
    o->nu_ta = o->nu_ta + o->co.nu;
    o->cd_ta = o->cd_ta + o->co.cd;
    o->cl_ta = o->cl_ta + cl;
    o->st_ta = o->st_ta + o->st;
    o->cpb_ta = o->cpb_ta + o->co.cpb;
    o->cl_amp_ta = o->cl_amp_ta + o->cl_amp;
    const double n = (double)o->niter_pos;
    const double dum_a = o->cd_ta / n, dum_b = o->cl_ta / n;
    o->rms_cd = o->rms_cd + (o->co.cd - dum_a) * (o->co.cd - dum_a);
    o->rms_cl = o->rms_cl + (cl - dum_b) * (cl - dum_b);
    orc_post *r = &o->post;
    r->time = rtime;
    r->nu = o->nu_ta / n;
    r->cd = dum_a;
    r->cl = dum_b;
    r->cl_amp = o->cl_amp_ta / n;
    r->cpb = o->cpb_ta / n;
    r->st = o->st_ta / n;
    r->rms_cd = sqrt(o->rms_cd / n);
    r->rms_cl = sqrt(o->rms_cl / n);
    r->st_last = o->st;
    r->cl_amp_last = o->cl_amp;
    r->niter = o->niter_pos;
}

const orc_post *orc_post_record(const orc *o) { return &o->post; }

/* POST_PROCESS, IPOST=1 branch (post_process.f90:19-36). */
void orc_post_final(orc *o, orc_post *out, double *u, double *v, double *p, double *t, double *vor)
{
    const double n = (double)o->niter_pos;
    for (int c = 0; c < o->n; c++) {
        if (u) u[c] = o->U_TA[c] / n;
        if (v) v[c] = o->V_TA[c] / n;
        if (p) p[c] = o->P_TA[c] / n;
        if (t) t[c] = o->T_TA[c] / n;
        if (vor) vor[c] = o->VOR_TA[c] / n;
    }
    if (out) {
        out->time = o->rtime;
        out->nu = o->nu_ta / n;
        out->cd = o->cd_ta / n;
        out->cl = o->cl_ta / n;
        out->st = o->st_ta / n;
        out->cpb = o->cpb_ta / n;
        out->cl_amp = o->cl_amp_ta / n;
        out->rms_cd = sqrt(o->rms_cd / n);
        out->rms_cl = sqrt(o->rms_cl / n);
        out->st_last = o->st;
        out->cl_amp_last = o->cl_amp;
        out->niter = o->niter_pos;
    }
}

/* CALCCOEF (calccoef.f90:9-120): CFL, base pressure, wall forces, Nusselt. */
void orc_calccoef(orc *o)
{
    const int NI = o->NI, NJ = o->NJ;
    const double pi = o->pi;
    double cfl = 0.0;
    for (int i = 1; i <= NI - 1; i++)
        for (int j = 1; j <= NJ - 1; j++) {
            int c = ID(i, j);
            double l = o->p.dt * (fabs(o->XIX[c] * o->U[c] + o->XIY[c] * o->V[c]) + fabs(o->ETX[c] * o->U[c] + o->ETY[c] * o->V[c]));
            cfl = fmax(cfl, l);
        }
    /* calccoef.f90:31-45.  The far-field node value PG(NI,NJ/2) is never
     * assigned during a run (WRITEDATA fills PG only every NITER_W=10^6 steps),
     * so the reference reads its zero initial value. */
    const double *P = o->P;
    double pg11 = 0.25 * (((P[ID(1, 1)] + P[ID(1, 0)]) + P[ID(0, 1)]) + P[ID(0, 0)]);
    double cpb = 2.0 * (0.0 - pg11);
    double p_drag = 0.0, p_lift = 0.0, t_drag = 0.0, t_lift = 0.0, sum_nu = 0.0;
    for (int j = 1; j <= NJ - 1; j++) { /* calccoef.f90:58-107 */
        int c = ID(1, j);
        double X = o->X[c], Y = o->Y[c];
        double xa = o->XG[ID(1, j)], ya = o->YG[ID(1, j)], xb = o->XG[ID(1, j + 1)], yb = o->YG[ID(1, j + 1)];
        double L1 = sqrt((X - xa) * (X - xa) + (Y - ya) * (Y - ya));
        double L2 = sqrt((X - xb) * (X - xb) + (Y - yb) * (Y - yb));
        double L3 = sqrt((xb - xa) * (xb - xa) + (yb - ya) * (yb - ya));
        double TH1 = acos((((L1 * L1) + (L2 * L2)) - (L3 * L3)) / ((2.0 * L1) * L2));
        double DN1 = ((L1 * L2) / L3) * sin(TH1);
        double LA = (yb - ya) / (xb - xa);
        double LB = ya - LA * xa;
        double LA_ = -1.0 / LA;
        double LB_ = Y - LA_ * X;
        double X1 = (LB_ - LB) / (LA - LA_);
        double Y1 = (LA * (LB_ - LB)) / (LA - LA_) + LB;
        double DN2 = sqrt((Y - Y1) * (Y - Y1) + (X - X1) * (X - X1));
        /* calccoef.f90:73-76 compares DN1 and DN2 and pauses; dropped */
        double TH2 = atan((Y - Y1) / (X - X1));
        double s = asin((Y - Y1) / DN2);
        if (TH2 >= 0.0 && s > 0.0) TH2 = TH2;
        else if (TH2 < 0.0 && s > 0.0) TH2 = pi + TH2;
        else if (TH2 >= 0.0 && s <= 0.0) TH2 = pi + TH2;
        else if (TH2 < 0.0 && s < 0.0) TH2 = 2.0 * pi + TH2;
        double dudn = ((o->U[c] * sin(TH2) - o->V[c] * cos(TH2)) - o->p.vel_rot) / DN1;
        double dtdn = (o->T[c] - o->p.t_wall) / DN1;
        double th = o->THETA[c], ar = o->AREA[c];
        p_drag = p_drag - ((2.0 * P[c]) * ar) * cos(th);
        p_lift = p_lift - ((2.0 * P[c]) * ar) * sin(th);
        t_drag = t_drag + (((2.0 / o->p.re) * dudn) * ar) * sin(th);
        t_lift = t_lift - (((2.0 / o->p.re) * dudn) * ar) * cos(th);
        sum_nu = sum_nu + dtdn * ar;
    }
    o->cl_nm1 = o->co.cl; /* calccoef.f90:109 */
    o->co.time = o->rtime;
    o->co.cfl = cfl;
    o->co.cpb = cpb;
    o->co.cd_p = p_drag;
    o->co.cl_p = p_lift;
    o->co.cd_v = t_drag;
    o->co.cl_v = t_lift;
    o->co.cd = p_drag + t_drag;
    o->co.cl = p_lift + t_lift;
    o->co.nu = -sum_nu / o->sum_area;
    if (o->ipost) post_step(o);
}

int orc_step(orc *o, int nsteps)
{
    if (!o) return -1;
    for (int s = 0; s < nsteps; s++) {
        orc_begin_step(o);
        orc_contra_vel(o);
        orc_explicit(o);
        orc_iter_u(o);
        orc_iter_v(o);
        orc_remove_grad(o);
        orc_iter_p(o);
        orc_correct(o);
        if (o->p.thermal) orc_iter_t(o);
        orc_calccoef(o);
        if (!isfinite(o->co.cd)) return -3;
    }
    return 0;
}

const orc_coeffs *orc_last_coeffs(const orc *o) { return &o->co; }
int orc_size(const orc *o) { return o->n; }
double orc_time(const orc *o) { return o->rtime; }
void orc_set_time(orc *o, double t, int niter) { o->rtime = t; o->niter_time = niter; }
double orc_sum_area(const orc *o) { return o->sum_area; }

double *orc_array(orc *o, const char *name)
{
    struct { const char *n; double *a; } t[] = {
        {"U", o->U}, {"V", o->V}, {"P", o->P}, {"T", o->T}, {"U_N", o->U_N}, {"V_N", o->V_N},
        {"T_N", o->T_N}, {"NLX", o->NLX}, {"NLY", o->NLY}, {"ADV", o->ADV}, {"NLX_NM1", o->NLX_NM1},
        {"NLY_NM1", o->NLY_NM1}, {"ADV_NM1", o->ADV_NM1}, {"DIFX", o->DIFX}, {"DIFY", o->DIFY},
        {"DIFT", o->DIFT}, {"S_U", o->S_U}, {"S_V", o->S_V}, {"UE", o->UE}, {"UW", o->UW},
        {"VN", o->VN}, {"VS", o->VS}, {"X", o->X}, {"Y", o->Y}, {"XG", o->XG}, {"YG", o->YG},
        {"XIX", o->XIX}, {"XIY", o->XIY}, {"ETX", o->ETX}, {"ETY", o->ETY}, {"DJAC", o->DJAC},
        {"Q11", o->Q11}, {"Q12", o->Q12}, {"Q22", o->Q22}, {"DE", o->DE}, {"DW", o->DW},
        {"DN", o->DN}, {"DS", o->DS}, {"THETA", o->THETA}, {"AREA", o->AREA}, {"AP", o->AP},
        {"AE", o->AE}, {"AW", o->AW}, {"AN", o->AN}, {"AS", o->AS}, {"SU", o->SU}, {"DD", o->DD},
        {"U1", o->U1}, {"U2", o->U2}, {"VOR", o->VOR}, {"U_TA", o->U_TA}, {"V_TA", o->V_TA},
        {"P_TA", o->P_TA}, {"T_TA", o->T_TA}, {"VOR_TA", o->VOR_TA}};
    for (size_t k = 0; k < sizeof(t) / sizeof(t[0]); k++)
        if (strcmp(t[k].n, name) == 0) return t[k].a;
    return NULL;
}
