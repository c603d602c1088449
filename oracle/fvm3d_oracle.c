/*
 * fvm3d_oracle.c -- CPU restatement of the reference's 3-D LES step (test
 * infrastructure only; see fvm3d_oracle.h).  Every routine cites the reference
 * file and lines it restates (LES/v2.3_LES-Reynolds stresses/).  Parity is
 * unpinned by the reference's own output (no Fortran compiler or MPI here).
 */
#include "fvm3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct o3 {
    o3_params p;
    int NI, NJ, NK, NI1, NJ1, n;
    double pi, pe, rtime, sum_area;
    int niter_time;
    /* geometry */
    double *XG, *YG, *ZG, *X, *Y, *Z;
    double *XIX, *XIY, *XIZ, *ETX, *ETY, *ETZ, *ZTX, *ZTY, *ZTZ, *DJAC;
    double *Q11, *Q12, *Q13, *Q22, *Q23, *Q33;
    double *DE, *DW, *DN, *DS, *DT, *DB, *THETA, *AREA1, *AREA2;
    /* state */
    double *U, *V, *W, *P, *T, *U_N, *V_N, *W_N, *T_N;
    double *NLX, *NLY, *NLZ, *ADV, *NLX_NM1, *NLY_NM1, *NLZ_NM1, *ADV_NM1;
    double *DIFX, *DIFY, *DIFZ, *DIFT, *S_U, *S_V, *S_W;
    /* fluxes, coefficients, scratch */
    double *U1, *U2, *U3, *UE, *UW, *VN, *VS, *WT, *WB;
    double *AP, *AE, *AW, *AN, *AS, *AT, *AB, *SU, *DD;
    /* LES */
    double *FW, *L[9], *DTD[3], *MAG, *UH, *VH, *WH, *TH, *MAGH, *DIN, *DOUT, *LIJ, *MIJ, *LM, *MM;
    double *EV, *EC, *SGSX, *SGSY, *SGSZ, *SGST;
    double *la, *lb, *lc, *ld, *lx, *lz, *lw, *lu, *lbb;
    /* post-processing sums (calccoef.f90:287-306): U, V, W, P, T, UU, UV, UW, VV, VW,
     * WW, SGS11, SGS12, SGS13, SGS22, SGS23, SGS33 */
    double *PS[17];
    int ipost, niter_pos;
    o3_coeffs co;
};

#define ID(i, j, k) ((i) + o->NI1 * ((j) + o->NJ1 * (k)))

static double *zalloc(size_t n) { return (double *)calloc(n, sizeof(double)); }

static double **fields(o3 *o, int *count)
{
    static double **list[128];
    int c = 0;
#define F(a) list[c++] = &o->a
    F(XG); F(YG); F(ZG); F(X); F(Y); F(Z);
    F(XIX); F(XIY); F(XIZ); F(ETX); F(ETY); F(ETZ); F(ZTX); F(ZTY); F(ZTZ); F(DJAC);
    F(Q11); F(Q12); F(Q13); F(Q22); F(Q23); F(Q33);
    F(DE); F(DW); F(DN); F(DS); F(DT); F(DB); F(THETA); F(AREA1); F(AREA2);
    F(U); F(V); F(W); F(P); F(T); F(U_N); F(V_N); F(W_N); F(T_N);
    F(NLX); F(NLY); F(NLZ); F(ADV); F(NLX_NM1); F(NLY_NM1); F(NLZ_NM1); F(ADV_NM1);
    F(DIFX); F(DIFY); F(DIFZ); F(DIFT); F(S_U); F(S_V); F(S_W);
    F(U1); F(U2); F(U3); F(UE); F(UW); F(VN); F(VS); F(WT); F(WB);
    F(AP); F(AE); F(AW); F(AN); F(AS); F(AT); F(AB); F(SU); F(DD);
    F(FW); F(L[0]); F(L[1]); F(L[2]); F(L[3]); F(L[4]); F(L[5]); F(L[6]); F(L[7]); F(L[8]);
    F(DTD[0]); F(DTD[1]); F(DTD[2]); F(MAG); F(UH); F(VH); F(WH); F(TH); F(MAGH);
    F(DIN); F(DOUT); F(LIJ); F(MIJ); F(LM); F(MM); F(EV); F(EC); F(SGSX); F(SGSY); F(SGSZ); F(SGST);
    for (int q = 0; q < 17; q++) F(PS[q]);
#undef F
    *count = c;
    return (double **)list;
}

o3 *o3_create(const o3_params *p)
{
    if (!p || p->ni < 6 || p->nj < 6 || p->nk < 6) return NULL;
    o3 *o = (o3 *)calloc(1, sizeof(o3));
    if (!o) return NULL;
    o->p = *p;
    if (o->p.res_every < 1) o->p.res_every = 1;
    o->NI = p->ni;
    o->NJ = p->nj;
    o->NK = p->nk;
    o->NI1 = p->ni + 1;
    o->NJ1 = p->nj + 1;
    o->n = (p->ni + 1) * (p->nj + 1) * (p->nk + 1);
    o->pi = 4.0 * atan(1.0);
    o->pe = p->re * p->pr;
    int cnt;
    double ***list = (double ***)fields(o, &cnt);
    for (int k = 0; k < cnt; k++) {
        *list[k] = zalloc((size_t)o->n);
        if (!*list[k]) { o3_destroy(o); return NULL; }
    }
    int m = (p->ni > p->nj ? p->ni : p->nj);
    m = (m > p->nk ? m : p->nk) + 2;
    o->la = zalloc(m); o->lb = zalloc(m); o->lc = zalloc(m); o->ld = zalloc(m); o->lx = zalloc(m);
    o->lz = zalloc(m); o->lw = zalloc(m); o->lu = zalloc(m); o->lbb = zalloc(m);
    return o;
}

void o3_destroy(o3 *o)
{
    if (!o) return;
    int cnt;
    double ***list = (double ***)fields(o, &cnt);
    for (int k = 0; k < cnt; k++) free(*list[k]);
    free(o->la); free(o->lb); free(o->lc); free(o->ld); free(o->lx);
    free(o->lz); free(o->lw); free(o->lu); free(o->lbb);
    free(o);
}

int o3_size(const o3 *o) { return o->n; }
const o3_coeffs *o3_last_coeffs(const o3 *o) { return &o->co; }

/* MPI_X (mpi_x.f90:25-51) for one periodic rank: J planes for every K, then K
 * planes for every J. */
static void halo(o3 *o, double *a)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    for (int k = 0; k <= NK; k++)
        for (int i = 0; i <= NI; i++) {
            a[ID(i, 0, k)] = a[ID(i, NJ - 1, k)];
            a[ID(i, NJ, k)] = a[ID(i, 1, k)];
        }
    for (int j = 0; j <= NJ; j++)
        for (int i = 0; i <= NI; i++) {
            a[ID(i, j, 0)] = a[ID(i, j, NK - 1)];
            a[ID(i, j, NK)] = a[ID(i, j, 1)];
        }
}

/* ------------------------------------------------------------------------- */
/* GRID: cell centres (grid.f90:75-320)                                      */
/* ------------------------------------------------------------------------- */
static void grid_centres(o3 *o)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    double *C[3] = {o->X, o->Y, o->Z};
    const double *G[3] = {o->XG, o->YG, o->ZG};
    for (int q = 0; q < 3; q++) {
        double *A = C[q];
        const double *g = G[q];
        for (int k = 1; k <= NK - 1; k++)
            for (int j = 1; j <= NJ - 1; j++)
                for (int i = 1; i <= NI - 1; i++)
                    A[ID(i, j, k)] = 0.125 * (((((((g[ID(i + 1, j + 1, k)] + g[ID(i + 1, j, k)]) + g[ID(i, j + 1, k)]) +
                                                  g[ID(i, j, k)]) + g[ID(i + 1, j + 1, k + 1)]) + g[ID(i + 1, j, k + 1)]) +
                                               g[ID(i, j + 1, k + 1)]) + g[ID(i, j, k + 1)]);
        /* boundary faces: face centre, then mirrored across the face */
        for (int k = 1; k <= NK - 1; k++)
            for (int j = 1; j <= NJ - 1; j++) {
                int i = 0;
                A[ID(i, j, k)] = 0.25 * (((g[ID(i + 1, j + 1, k)] + g[ID(i + 1, j, k)]) + g[ID(i + 1, j + 1, k + 1)]) +
                                         g[ID(i + 1, j, k + 1)]);
                A[ID(i, j, k)] = A[ID(i, j, k)] - (A[ID(i + 1, j, k)] - A[ID(i, j, k)]);
                i = NI;
                A[ID(i, j, k)] = 0.25 * (((g[ID(i, j + 1, k)] + g[ID(i, j, k)]) + g[ID(i, j + 1, k + 1)]) + g[ID(i, j, k + 1)]);
                A[ID(i, j, k)] = A[ID(i, j, k)] + (A[ID(i, j, k)] - A[ID(i - 1, j, k)]);
            }
        for (int k = 1; k <= NK - 1; k++)
            for (int i = 1; i <= NI - 1; i++) {
                int j = 0;
                A[ID(i, j, k)] = 0.25 * (((g[ID(i + 1, j + 1, k + 1)] + g[ID(i + 1, j + 1, k)]) + g[ID(i, j + 1, k + 1)]) +
                                         g[ID(i, j + 1, k)]);
                A[ID(i, j, k)] = A[ID(i, j, k)] - (A[ID(i, j + 1, k)] - A[ID(i, j, k)]);
                j = NJ;
                A[ID(i, j, k)] = 0.25 * (((g[ID(i + 1, j, k + 1)] + g[ID(i + 1, j, k)]) + g[ID(i, j, k + 1)]) + g[ID(i, j, k)]);
                A[ID(i, j, k)] = A[ID(i, j, k)] - (A[ID(i, j - 1, k)] - A[ID(i, j, k)]);
            }
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                int k = 0;
                A[ID(i, j, k)] = 0.25 * (((g[ID(i, j, k + 1)] + g[ID(i + 1, j, k + 1)]) + g[ID(i + 1, j + 1, k + 1)]) +
                                         g[ID(i, j + 1, k + 1)]);
                A[ID(i, j, k)] = A[ID(i, j, k)] - (A[ID(i, j, k + 1)] - A[ID(i, j, k)]);
                k = NK;
                A[ID(i, j, k)] = 0.25 * (((g[ID(i, j, k)] + g[ID(i + 1, j, k)]) + g[ID(i + 1, j + 1, k)]) + g[ID(i, j + 1, k)]);
                A[ID(i, j, k)] = A[ID(i, j, k)] + (A[ID(i, j, k)] - A[ID(i, j, k - 1)]);
            }
        halo(o, A);   /* grid.f90:255-259 */
    }
    /* spanwise end planes (grid.f90:261-320): x, y copied, z mirrored */
    for (int side = 0; side < 2; side++) {
        const int k = side ? NK : 0, kin = side ? NK - 1 : 1;
        for (int j = 0; j <= NJ; j++)
            for (int i = 0; i <= NI; i++) {
                o->X[ID(i, j, k)] = o->X[ID(i, j, kin)];
                o->Y[ID(i, j, k)] = o->Y[ID(i, j, kin)];
            }
        double *Zc = o->Z;
        const double *zg = o->ZG;
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                if (!side) {
                    Zc[ID(i, j, k)] = 0.25 * (((zg[ID(i, j, k + 1)] + zg[ID(i + 1, j, k + 1)]) + zg[ID(i + 1, j + 1, k + 1)]) +
                                              zg[ID(i, j + 1, k + 1)]);
                    Zc[ID(i, j, k)] = Zc[ID(i, j, k)] - (Zc[ID(i, j, k + 1)] - Zc[ID(i, j, k)]);
                } else {
                    Zc[ID(i, j, k)] = 0.25 * (((zg[ID(i, j, k)] + zg[ID(i + 1, j, k)]) + zg[ID(i + 1, j + 1, k)]) + zg[ID(i, j + 1, k)]);
                    Zc[ID(i, j, k)] = Zc[ID(i, j, k)] + (Zc[ID(i, j, k)] - Zc[ID(i, j, k - 1)]);
                }
            }
        for (int j = 1; j <= NJ - 1; j++) {
            Zc[ID(0, j, k)] = Zc[ID(1, j, k)];
            Zc[ID(NI, j, k)] = Zc[ID(NI - 1, j, k)];
        }
        for (int i = 1; i <= NI - 1; i++) {
            Zc[ID(i, 0, k)] = Zc[ID(i, 1, k)];
            Zc[ID(i, NJ, k)] = Zc[ID(i, NJ - 1, k)];
        }
        Zc[ID(0, 0, k)] = Zc[ID(1, 1, k)];
        Zc[ID(NI, 0, k)] = Zc[ID(NI - 1, 1, k)];
        Zc[ID(NI, NJ, k)] = Zc[ID(NI - 1, NJ - 1, k)];
        Zc[ID(0, NJ, k)] = Zc[ID(1, NJ - 1, k)];
    }
}

/* ------------------------------------------------------------------------- */
/* METRIC (metric.f90:33-520)                                                */
/* ------------------------------------------------------------------------- */
/* d/d(index) along direction dir at (i,j,k): central differences inside,
 * second-order one-sided on the domain boundary planes of that direction. */
static double dref(const o3 *o, const double *A, int i, int j, int k, int dir)
{
    const int lo = 0, hi = dir == 0 ? o->NI : (dir == 1 ? o->NJ : o->NK);
    const int q = dir == 0 ? i : (dir == 1 ? j : k);
    const int si = dir == 0, sj = dir == 1, sk = dir == 2;
#define AT(s) A[ID(i + (s) * si, j + (s) * sj, k + (s) * sk)]
    if (q == lo) return ((-3.0 * AT(0) + 4.0 * AT(1)) - AT(2)) / 2.0;
    if (q == hi) return ((3.0 * AT(0) - 4.0 * AT(-1)) + AT(-2)) / 2.0;
    return 0.5 * (AT(1) - AT(-1));
#undef AT
}

static int metric(o3 *o)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK, n = o->n;
    double *d[9];
    for (int q = 0; q < 9; q++) {
        d[q] = zalloc((size_t)n);
        if (!d[q]) { for (int r = 0; r < q; r++) free(d[r]); return -1; }
    }
    /* XXI XET XZT YXI YET YZT ZXI ZET ZZT */
    const double *C[3] = {o->X, o->Y, o->Z};
    for (int k = 0; k <= NK; k++)
        for (int j = 0; j <= NJ; j++)
            for (int i = 0; i <= NI; i++)
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) d[3 * a + b][ID(i, j, k)] = dref(o, C[a], i, j, k, b);
    for (int q = 0; q < 9; q++) halo(o, d[q]);   /* metric.f90:400-412 */
    double *XXI = d[0], *XET = d[1], *XZT = d[2], *YXI = d[3], *YET = d[4], *YZT = d[5], *ZXI = d[6], *ZET = d[7],
           *ZZT = d[8];
    for (int c = 0; c < n; c++) {
        double J = (XXI[c] * (YET[c] * ZZT[c] - YZT[c] * ZET[c]) - YXI[c] * (XET[c] * ZZT[c] - ZET[c] * XZT[c])) +
                   ZXI[c] * (XET[c] * YZT[c] - XZT[c] * YET[c]);
        o->DJAC[c] = J;
        o->XIX[c] = (YET[c] * ZZT[c] - YZT[c] * ZET[c]) / J;
        o->XIY[c] = (ZET[c] * XZT[c] - ZZT[c] * XET[c]) / J;
        o->XIZ[c] = (XET[c] * YZT[c] - XZT[c] * YET[c]) / J;
        o->ETX[c] = (YZT[c] * ZXI[c] - YXI[c] * ZZT[c]) / J;
        o->ETY[c] = (ZZT[c] * XXI[c] - ZXI[c] * XZT[c]) / J;
        o->ETZ[c] = (XZT[c] * YXI[c] - XXI[c] * YZT[c]) / J;
        o->ZTX[c] = (YXI[c] * ZET[c] - YET[c] * ZXI[c]) / J;
        o->ZTY[c] = (ZXI[c] * XET[c] - ZET[c] * XXI[c]) / J;
        o->ZTZ[c] = (XXI[c] * YET[c] - XET[c] * YXI[c]) / J;
    }
    for (int q = 0; q < 9; q++) free(d[q]);
    for (int c = 0; c < n; c++) {
        o->Q11[c] = (o->XIX[c] * o->XIX[c] + o->XIY[c] * o->XIY[c]) + o->XIZ[c] * o->XIZ[c];
        o->Q12[c] = (o->XIX[c] * o->ETX[c] + o->XIY[c] * o->ETY[c]) + o->XIZ[c] * o->ETZ[c];
        o->Q13[c] = (o->ZTX[c] * o->XIX[c] + o->ZTY[c] * o->XIY[c]) + o->ZTZ[c] * o->XIZ[c];
        o->Q22[c] = (o->ETX[c] * o->ETX[c] + o->ETY[c] * o->ETY[c]) + o->ETZ[c] * o->ETZ[c];
        o->Q23[c] = (o->ETX[c] * o->ZTX[c] + o->ETY[c] * o->ZTY[c]) + o->ETZ[c] * o->ZTZ[c];
        o->Q33[c] = (o->ZTX[c] * o->ZTX[c] + o->ZTY[c] * o->ZTY[c]) + o->ZTZ[c] * o->ZTZ[c];
    }
    const double *J = o->DJAC;
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                int c = ID(i, j, k);
                o->DE[c] = 0.5 * (J[c] * o->Q11[c] + J[ID(i + 1, j, k)] * o->Q11[ID(i + 1, j, k)]);
                o->DW[c] = 0.5 * (J[c] * o->Q11[c] + J[ID(i - 1, j, k)] * o->Q11[ID(i - 1, j, k)]);
                o->DN[c] = 0.5 * (J[c] * o->Q22[c] + J[ID(i, j + 1, k)] * o->Q22[ID(i, j + 1, k)]);
                o->DS[c] = 0.5 * (J[c] * o->Q22[c] + J[ID(i, j - 1, k)] * o->Q22[ID(i, j - 1, k)]);
                o->DT[c] = 0.5 * (J[c] * o->Q33[c] + J[ID(i, j, k + 1)] * o->Q33[ID(i, j, k + 1)]);
                o->DB[c] = 0.5 * (J[c] * o->Q33[c] + J[ID(i, j, k - 1)] * o->Q33[ID(i, j, k - 1)]);
            }
    for (int c = 0; c < n; c++)
        if (!(fabs(o->DJAC[c]) >= 1e-15)) return -2;
    return 0;
}

int o3_set_grid(o3 *o, const double *xg, const double *yg, const double *zg)
{
    if (!o || !xg || !yg || !zg) return -1;
    memcpy(o->XG, xg, sizeof(double) * (size_t)o->n);
    memcpy(o->YG, yg, sizeof(double) * (size_t)o->n);
    memcpy(o->ZG, zg, sizeof(double) * (size_t)o->n);
    grid_centres(o);
    return metric(o);
}

/* ------------------------------------------------------------------------- */
/* INIT (init.f90:150-200): uniform flow, THETA, wall face areas               */
/* ------------------------------------------------------------------------- */
int o3_init(o3 *o, const double *du, const double *dv, const double *dw)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK, n = o->n;
    const double pi = o->pi;
    for (int c = 0; c < n; c++) {
        o->U[c] = 1.0; o->V[c] = 0.0; o->W[c] = 0.0; o->T[c] = 0.0; o->P[c] = 0.0;
        o->NLX[c] = o->NLY[c] = o->NLZ[c] = o->ADV[c] = 0.0;
    }
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                int c = ID(i, j, k);
                if (du) o->U[c] += du[c];
                if (dv) o->V[c] += dv[c];
                if (dw) o->W[c] += dw[c];
            }
    for (int c = 0; c < n; c++) {
        double R = sqrt(o->X[c] * o->X[c] + o->Y[c] * o->Y[c]);
        double th = atan(o->Y[c] / o->X[c]);
        double s = asin(o->Y[c] / R);
        if (th >= 0.0 && s > 0.0) th = th;
        else if (th < 0.0 && s > 0.0) th = pi + th;
        else if (th >= 0.0 && s <= 0.0) th = pi + th;
        else if (th < 0.0 && s < 0.0) th = 2.0 * pi + th;
        o->THETA[c] = th;
    }
    const double *XG = o->XG, *YG = o->YG, *ZG = o->ZG;
    double dum = 0.0;
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++) {
            const int i = 1;
#define DX(a, b) (XG[a] - XG[b])
#define DY(a, b) (YG[a] - YG[b])
#define DZ(a, b) (ZG[a] - ZG[b])
#define LEN(a, b) sqrt((DX(a, b) * DX(a, b) + DY(a, b) * DY(a, b)) + DZ(a, b) * DZ(a, b))
            int p00 = ID(i, j, k), p10 = ID(i, j + 1, k), p01 = ID(i, j, k + 1), p11 = ID(i, j + 1, k + 1);
            double L1 = LEN(p10, p00), L2 = LEN(p01, p00), L3 = LEN(p10, p01);
            double TH1 = acos(((L3 * L3 - L2 * L2) - L1 * L1) / ((-2.0 * L1) * L2));
            o->AREA1[ID(i, j, k)] = ((0.5 * L1) * L2) * sin(TH1);
            L1 = LEN(p11, p10);
            L2 = LEN(p11, p01);
            TH1 = acos(((L3 * L3 - L2 * L2) - L1 * L1) / ((-2.0 * L1) * L2));
            o->AREA2[ID(i, j, k)] = ((0.5 * L1) * L2) * sin(TH1);
            dum = (dum + o->AREA1[ID(i, j, k)]) + o->AREA2[ID(i, j, k)];
#undef DX
#undef DY
#undef DZ
#undef LEN
        }
    o->sum_area = dum;
    o->rtime = 0.0;
    o->niter_time = 0;
    memset(&o->co, 0, sizeof(o->co));
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Boundary conditions                                                        */
/* ------------------------------------------------------------------------- */
/* BCU / BCT (bcu.f90:14-48, bct.f90): wall Dirichlet by ghost (U_F = 0 for the
 * velocities, T_WALL for T) folded into AP/SU/AW, far field inflow value or the
 * convective outflow value from the step-n field, folded into AP/SU/AE, then the
 * periodic copy.  kind: 0 U, 1 V or W, 2 T. */
static void bc_field(o3 *o, int kind, double *A, const double *B)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    const double pi = o->pi;
    const double uf = kind == 2 ? o->p.t_wall : 0.0;
    for (int k = 0; k <= NK; k++)
        for (int j = 0; j <= NJ; j++) {
            int c = ID(1, j, k);
            o->AP[c] = o->AP[c] + o->AW[c];
            o->SU[c] = o->SU[c] + (2.0 * o->AW[c]) * uf;
            o->AW[c] = 0.0;
            A[ID(0, j, k)] = (-A[c]) + 2.0 * uf;
        }
    const double fin = kind == 0 ? 1.0 : (kind == 1 ? 0.0 : o->p.tin);
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++) {
            const int i = NI;
            double f;
            double th = o->THETA[ID(i, j, k)];
            if (th >= 0.5 * pi && th <= 1.5 * pi) {
                f = fin;
            } else {
                f = 0.5 * (B[ID(i, j, k)] + B[ID(i - 1, j, k)]) -
                    (o->p.dt * 1.0) *
                        ((0.5 * (o->XIX[ID(i, j, k)] + o->XIX[ID(i - 1, j, k)]) * (B[ID(i, j, k)] - B[ID(i - 1, j, k)]) +
                          (0.5 * (o->ETX[ID(i, j, k)] + o->ETX[ID(i - 1, j, k)]) * 0.25) *
                              (((B[ID(i, j + 1, k)] + B[ID(i - 1, j + 1, k)]) - B[ID(i, j - 1, k)]) - B[ID(i - 1, j - 1, k)])) +
                         (0.5 * (o->ZTX[ID(i, j, k)] + o->ZTX[ID(i - 1, j, k)]) * 0.25) *
                             (((B[ID(i, j, k + 1)] + B[ID(i - 1, j, k + 1)]) - B[ID(i, j, k - 1)]) - B[ID(i - 1, j, k - 1)]));
            }
            int cm = ID(NI - 1, j, k);
            o->AP[cm] = o->AP[cm] + o->AE[cm];
            o->SU[cm] = o->SU[cm] + (2.0 * o->AE[cm]) * f;
            o->AE[cm] = 0.0;
            A[ID(i, j, k)] = (-A[ID(i - 1, j, k)]) + 2.0 * f;
        }
    halo(o, A);
}

/* BCP (bcp.f90:22-36): Neumann wall (AP -= AW, AW = 0, P0 = P1), far field
 * AE(NI-1) = 0 and cubic extrapolation, periodic copy. */
static void bcp(o3 *o)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    double *P = o->P;
    for (int k = 0; k <= NK; k++)
        for (int j = 1; j <= NJ - 1; j++) {
            int c = ID(1, j, k);
            o->AP[c] = o->AP[c] - o->AW[c];
            o->AW[c] = 0.0;
            P[ID(0, j, k)] = P[c];
            o->AE[ID(NI - 1, j, k)] = 0.0;
            P[ID(NI, j, k)] = (3.0 * P[ID(NI - 1, j, k)] - 3.0 * P[ID(NI - 2, j, k)]) + P[ID(NI - 3, j, k)];
        }
    halo(o, P);
}

/* ------------------------------------------------------------------------- */
/* Explicit operators                                                          */
/* ------------------------------------------------------------------------- */
/* CONTRA_VEL (contra_vel.f90:13-53) */
static void contra_vel(o3 *o)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK, n = o->n;
    for (int c = 0; c < n; c++) {
        o->U1[c] = (o->XIX[c] * o->U[c] + o->XIY[c] * o->V[c]) + o->XIZ[c] * o->W[c];
        o->U2[c] = (o->ETX[c] * o->U[c] + o->ETY[c] * o->V[c]) + o->ETZ[c] * o->W[c];
        o->U3[c] = (o->ZTX[c] * o->U[c] + o->ZTY[c] * o->V[c]) + o->ZTZ[c] * o->W[c];
    }
    halo(o, o->U1);
    halo(o, o->U2);
    halo(o, o->U3);
    const double *J = o->DJAC;
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                int c = ID(i, j, k);
                o->UE[c] = 0.5 * (J[c] * o->U1[c] + J[ID(i + 1, j, k)] * o->U1[ID(i + 1, j, k)]);
                o->UW[c] = 0.5 * (J[c] * o->U1[c] + J[ID(i - 1, j, k)] * o->U1[ID(i - 1, j, k)]);
                o->VN[c] = 0.5 * (J[c] * o->U2[c] + J[ID(i, j + 1, k)] * o->U2[ID(i, j + 1, k)]);
                o->VS[c] = 0.5 * (J[c] * o->U2[c] + J[ID(i, j - 1, k)] * o->U2[ID(i, j - 1, k)]);
                o->WT[c] = 0.5 * (J[c] * o->U3[c] + J[ID(i, j, k + 1)] * o->U3[ID(i, j, k + 1)]);
                o->WB[c] = 0.5 * (J[c] * o->U3[c] + J[ID(i, j, k - 1)] * o->U3[ID(i, j, k - 1)]);
            }
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++) o->UW[ID(1, j, k)] = 0.0;
}

/* NL (nl.f90:23-31) */
static void nl(o3 *o, const double *in, double *out)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                int c = ID(i, j, k);
                double p = in[c];
                out[c] = 0.5 * ((((((o->UE[c] * (in[ID(i + 1, j, k)] + p) - o->UW[c] * (in[ID(i - 1, j, k)] + p)) +
                                    o->VN[c] * (in[ID(i, j + 1, k)] + p)) - o->VS[c] * (in[ID(i, j - 1, k)] + p)) +
                                  o->WT[c] * (in[ID(i, j, k + 1)] + p)) - o->WB[c] * (in[ID(i, j, k - 1)] + p)));
            }
}

/* DIF_DIAGONAL (dif_diagonal.f90:13-32): the twelve cross-derivative terms */
static double cross12(const o3 *o, const double *f, int i, int j, int k)
{
    const double *J = o->DJAC;
#define F(a, b, c) f[ID(i + (a), j + (b), k + (c))]
#define G(Q, a, b, c) (o->Q[ID(i + (a), j + (b), k + (c))] * J[ID(i + (a), j + (b), k + (c))])
    double s = G(Q12, 1, 0, 0) * (F(1, 1, 0) - F(1, -1, 0));
    s = s - G(Q12, -1, 0, 0) * (F(-1, 1, 0) - F(-1, -1, 0));
    s = s + G(Q13, 1, 0, 0) * (F(1, 0, 1) - F(1, 0, -1));
    s = s - G(Q13, -1, 0, 0) * (F(-1, 0, 1) - F(-1, 0, -1));
    s = s + G(Q12, 0, 1, 0) * (F(1, 1, 0) - F(-1, 1, 0));
    s = s - G(Q12, 0, -1, 0) * (F(1, -1, 0) - F(-1, -1, 0));
    s = s + G(Q23, 0, 1, 0) * (F(0, 1, 1) - F(0, 1, -1));
    s = s - G(Q23, 0, -1, 0) * (F(0, -1, 1) - F(0, -1, -1));
    s = s + G(Q13, 0, 0, 1) * (F(1, 0, 1) - F(-1, 0, 1));
    s = s - G(Q13, 0, 0, -1) * (F(1, 0, -1) - F(-1, 0, -1));
    s = s + G(Q23, 0, 0, 1) * (F(0, 1, 1) - F(0, -1, 1));
    s = s - G(Q23, 0, 0, -1) * (F(0, 1, -1) - F(0, -1, -1));
#undef F
#undef G
    return 0.25 * s;
}

static void dif_diagonal(o3 *o, const double *f, double *out)
{
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) out[ID(i, j, k)] = cross12(o, f, i, j, k);
}

/* DIF (dif.f90:15-23) */
static void dif(o3 *o, const double *in, double *out)
{
    dif_diagonal(o, in, o->DD);
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) {
                int c = ID(i, j, k);
                double p = in[c];
                out[c] = 1.0 * ((((((o->DE[c] * (in[ID(i + 1, j, k)] - p) + o->DW[c] * (in[ID(i - 1, j, k)] - p)) +
                                    o->DN[c] * (in[ID(i, j + 1, k)] - p)) + o->DS[c] * (in[ID(i, j - 1, k)] - p)) +
                                  o->DT[c] * (in[ID(i, j, k + 1)] - p)) + o->DB[c] * (in[ID(i, j, k - 1)] - p)) +
                                o->DD[c]);
            }
}

/* P_SOURCE (p_source.f90:14-42) */
static void p_source(o3 *o, const double *in)
{
    const double *J = o->DJAC;
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) {
                int c = ID(i, j, k), e = ID(i + 1, j, k), w = ID(i - 1, j, k), nn = ID(i, j + 1, k), s = ID(i, j - 1, k),
                    t = ID(i, j, k + 1), b = ID(i, j, k - 1);
                const double *M1[3] = {o->XIX, o->XIY, o->XIZ}, *M2[3] = {o->ETX, o->ETY, o->ETZ},
                             *M3[3] = {o->ZTX, o->ZTY, o->ZTZ};
                double *out[3] = {o->S_U, o->S_V, o->S_W};
                for (int q = 0; q < 3; q++) {
                    double a = (((((J[e] * M1[q][e]) * in[e] - (J[w] * M1[q][w]) * in[w]) + (J[nn] * M2[q][nn]) * in[nn]) -
                                 (J[s] * M2[q][s]) * in[s]) + (J[t] * M3[q][t]) * in[t]) - (J[b] * M3[q][b]) * in[b];
                    out[q][c] = -0.5 * a;
                }
            }
}

/* ------------------------------------------------------------------------- */
/* Line solves                                                                 */
/* ------------------------------------------------------------------------- */
static int jw(const o3 *o, int j) { return j == 0 ? o->NJ - 1 : (j == o->NJ ? 1 : j); }
static int kw(const o3 *o, int k) { return k == 0 ? o->NK - 1 : (k == o->NK ? 1 : k); }

/* Tridiagonal a x(e-1) + b x(e) + c x(e+1) = d, a[0] = c[n-1] = 0 (Thomas). */
static void thomas(int n, const double *a, const double *b, const double *c, const double *d, double *x, double *B)
{
    double Bprev = 0.0, xprev = 0.0;
    for (int e = 0; e < n; e++) {
        double D = b[e] - a[e] * Bprev;
        B[e] = c[e] / D;
        x[e] = (d[e] - a[e] * xprev) / D;
        Bprev = B[e];
        xprev = x[e];
    }
    for (int e = n - 2; e >= 0; e--) x[e] = x[e] - B[e] * x[e + 1];
}

/* Cyclic tridiagonal (a[0] couples x[n-1], c[n-1] couples x[0]) by
 * Sherman-Morrison with gamma = -b[0]. */
static void cyclic(int n, const double *a, const double *b, const double *c, const double *d, double *x, double *bb,
                   double *u, double *z, double *B)
{
    double gamma = -b[0], alpha = c[n - 1], beta = a[0];
    for (int e = 0; e < n; e++) bb[e] = b[e];
    bb[0] = b[0] - gamma;
    bb[n - 1] = b[n - 1] - alpha * beta / gamma;
    double a0 = a[0], cn = c[n - 1];
    double *aa = (double *)a, *cc = (double *)c;
    aa[0] = 0.0;
    cc[n - 1] = 0.0;
    thomas(n, aa, bb, cc, d, x, B);
    for (int e = 0; e < n; e++) u[e] = 0.0;
    u[0] = gamma;
    u[n - 1] = alpha;
    thomas(n, aa, bb, cc, u, z, B);
    aa[0] = a0;
    cc[n - 1] = cn;
    double fact = (x[0] + beta * x[n - 1] / gamma) / ((1.0 + z[0]) + beta * z[n - 1] / gamma);
    for (int e = 0; e < n; e++) x[e] = x[e] - fact * z[e];
}

/* One sweep of line solves along direction dir (0: I, 1: J, 2: K) for the field
 * phi with the coefficient arrays of the object.  Faithful: lexicographic order,
 * the reference's recurrences with lagged periodic ghosts (iter_u.f90:100-116,
 * 178-194, 255-271, lisolv.f90:21-38).  GPU order: red-black lines (colour =
 * parity of the transverse index sum), neighbours by periodic wrap, J and K
 * lines cyclic. */
static void sweep(o3 *o, int dir, double *phi, int cyclic_lines)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    double *A = o->la, *B = o->lb, *C = o->lc, *D = o->ld;
    if (o->p.order == O3_FAITHFUL) {
        if (dir == 0) {
            for (int k = 1; k <= NK - 1; k++)
                for (int j = 1; j <= NJ - 1; j++) {
                    for (int i = 1; i <= NI - 1; i++) {
                        int c = ID(i, j, k);
                        A[i] = -o->AW[c];
                        D[i] = o->AP[c] - A[i] * B[i - 1];
                        B[i] = -o->AE[c] / D[i];
                        C[i] = (((o->AN[c] * phi[ID(i, j + 1, k)] + o->AS[c] * phi[ID(i, j - 1, k)]) +
                                 o->AT[c] * phi[ID(i, j, k + 1)]) + o->AB[c] * phi[ID(i, j, k - 1)]) + o->SU[c];
                        phi[c] = (C[i] - A[i] * phi[ID(i - 1, j, k)]) / D[i];
                    }
                    for (int i = NI - 1; i >= 1; i--) phi[ID(i, j, k)] = phi[ID(i, j, k)] - B[i] * phi[ID(i + 1, j, k)];
                }
        } else if (dir == 1) {
            for (int k = 1; k <= NK - 1; k++)
                for (int i = 1; i <= NI - 1; i++) {
                    for (int j = 1; j <= NJ - 1; j++) {
                        int c = ID(i, j, k);
                        A[j] = -o->AS[c];
                        D[j] = o->AP[c] - A[j] * B[j - 1];
                        B[j] = -o->AN[c] / D[j];
                        C[j] = (((o->AE[c] * phi[ID(i + 1, j, k)] + o->AW[c] * phi[ID(i - 1, j, k)]) +
                                 o->AT[c] * phi[ID(i, j, k + 1)]) + o->AB[c] * phi[ID(i, j, k - 1)]) + o->SU[c];
                        phi[c] = (C[j] - A[j] * phi[ID(i, j - 1, k)]) / D[j];
                    }
                    for (int j = NJ - 1; j >= 1; j--) phi[ID(i, j, k)] = phi[ID(i, j, k)] - B[j] * phi[ID(i, j + 1, k)];
                }
        } else {
            for (int j = 1; j <= NJ - 1; j++)
                for (int i = 1; i <= NI - 1; i++) {
                    for (int k = 1; k <= NK - 1; k++) {
                        int c = ID(i, j, k);
                        A[k] = -o->AB[c];
                        D[k] = o->AP[c] - A[k] * B[k - 1];
                        B[k] = -o->AT[c] / D[k];
                        C[k] = (((o->AE[c] * phi[ID(i + 1, j, k)] + o->AW[c] * phi[ID(i - 1, j, k)]) +
                                 o->AN[c] * phi[ID(i, j + 1, k)]) + o->AS[c] * phi[ID(i, j - 1, k)]) + o->SU[c];
                        phi[c] = (C[k] - A[k] * phi[ID(i, j, k - 1)]) / D[k];
                    }
                    for (int k = NK - 1; k >= 1; k--) phi[ID(i, j, k)] = phi[ID(i, j, k)] - B[k] * phi[ID(i, j, k + 1)];
                }
        }
        return;
    }
    /* GPU order */
    double *a = o->la, *b = o->lb, *cc = o->lc, *d = o->ld, *x = o->lx;
    for (int colour = 0; colour < 2; colour++) {
        if (dir == 0) {
            for (int k = 1; k <= NK - 1; k++)
                for (int j = 1; j <= NJ - 1; j++) {
                    if (((j + k) & 1) != colour) continue;
                    const int n = NI - 1;
                    for (int e = 0; e < n; e++) {
                        int i = e + 1, c = ID(i, j, k);
                        a[e] = -o->AW[c];
                        b[e] = o->AP[c];
                        cc[e] = -o->AE[c];
                        d[e] = (((o->AN[c] * phi[ID(i, jw(o, j + 1), k)] + o->AS[c] * phi[ID(i, jw(o, j - 1), k)]) +
                                 o->AT[c] * phi[ID(i, j, kw(o, k + 1))]) + o->AB[c] * phi[ID(i, j, kw(o, k - 1))]) + o->SU[c];
                    }
                    a[0] = 0.0;
                    cc[n - 1] = 0.0;
                    thomas(n, a, b, cc, d, x, o->lz);
                    for (int e = 0; e < n; e++) phi[ID(e + 1, j, k)] = x[e];
                }
        } else if (dir == 1) {
            for (int k = 1; k <= NK - 1; k++)
                for (int i = 1; i <= NI - 1; i++) {
                    if (((i + k) & 1) != colour) continue;
                    const int n = NJ - 1;
                    for (int e = 0; e < n; e++) {
                        int j = e + 1, c = ID(i, j, k);
                        a[e] = -o->AS[c];
                        b[e] = o->AP[c];
                        cc[e] = -o->AN[c];
                        d[e] = (((o->AE[c] * phi[ID(i + 1, j, k)] + o->AW[c] * phi[ID(i - 1, j, k)]) +
                                 o->AT[c] * phi[ID(i, j, kw(o, k + 1))]) + o->AB[c] * phi[ID(i, j, kw(o, k - 1))]) + o->SU[c];
                    }
                    if (cyclic_lines) cyclic(n, a, b, cc, d, x, o->lbb, o->lu, o->lw, o->lz);
                    else { a[0] = 0.0; cc[n - 1] = 0.0; thomas(n, a, b, cc, d, x, o->lz); }
                    for (int e = 0; e < n; e++) phi[ID(i, e + 1, k)] = x[e];
                }
        } else {
            for (int j = 1; j <= NJ - 1; j++)
                for (int i = 1; i <= NI - 1; i++) {
                    if (((i + j) & 1) != colour) continue;
                    const int n = NK - 1;
                    for (int e = 0; e < n; e++) {
                        int k = e + 1, c = ID(i, j, k);
                        a[e] = -o->AB[c];
                        b[e] = o->AP[c];
                        cc[e] = -o->AT[c];
                        d[e] = (((o->AE[c] * phi[ID(i + 1, j, k)] + o->AW[c] * phi[ID(i - 1, j, k)]) +
                                 o->AN[c] * phi[ID(i, jw(o, j + 1), k)]) + o->AS[c] * phi[ID(i, jw(o, j - 1), k)]) + o->SU[c];
                    }
                    if (cyclic_lines) cyclic(n, a, b, cc, d, x, o->lbb, o->lu, o->lw, o->lz);
                    else { a[0] = 0.0; cc[n - 1] = 0.0; thomas(n, a, b, cc, d, x, o->lz); }
                    for (int e = 0; e < n; e++) phi[ID(i, j, e + 1)] = x[e];
                }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* ITER_U / ITER_T (iter_u.f90:23-255, iter_T.f90): three AF sweeps            */
/* ------------------------------------------------------------------------- */
static void af_coef(o3 *o, int split, double rek)
{
    const double *J = o->DJAC;
    const double *m1 = split == 0 ? o->XIX : (split == 1 ? o->XIY : o->XIZ);
    const double *m2 = split == 0 ? o->ETX : (split == 1 ? o->ETY : o->ETZ);
    const double *m3 = split == 0 ? o->ZTX : (split == 1 ? o->ZTY : o->ZTZ);
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) {
                int c = ID(i, j, k), e = ID(i + 1, j, k), w = ID(i - 1, j, k), nn = ID(i, j + 1, k), s = ID(i, j - 1, k),
                    t = ID(i, j, k + 1), b = ID(i, j, k - 1);
                o->AE[c] = 0.5 * (J[c] * (m1[c] * m1[c]) + J[e] * (m1[e] * m1[e]));
                o->AW[c] = 0.5 * (J[c] * (m1[c] * m1[c]) + J[w] * (m1[w] * m1[w]));
                o->AN[c] = 0.5 * (J[c] * (m2[c] * m2[c]) + J[nn] * (m2[nn] * m2[nn]));
                o->AS[c] = 0.5 * (J[c] * (m2[c] * m2[c]) + J[s] * (m2[s] * m2[s]));
                o->AT[c] = 0.5 * (J[c] * (m3[c] * m3[c]) + J[t] * (m3[t] * m3[t]));
                o->AB[c] = 0.5 * (J[c] * (m3[c] * m3[c]) + J[b] * (m3[b] * m3[b]));
                o->AP[c] = (((((((2.0 * rek) * J[c]) / o->p.dt + o->AE[c]) + o->AW[c]) + o->AN[c]) + o->AS[c]) + o->AT[c]) +
                           o->AB[c];
            }
}

/* Twelve cross terms of one AF factor (iter_u.f90:44-68) with the split's
 * metric products J*m_a*m_b. */
static double af_cross(const o3 *o, int split, const double *f, int i, int j, int k)
{
    const double *J = o->DJAC;
    const double *m1 = split == 0 ? o->XIX : (split == 1 ? o->XIY : o->XIZ);
    const double *m2 = split == 0 ? o->ETX : (split == 1 ? o->ETY : o->ETZ);
    const double *m3 = split == 0 ? o->ZTX : (split == 1 ? o->ZTY : o->ZTZ);
#define F(a, b, c) f[ID(i + (a), j + (b), k + (c))]
#define P3(ma, mb, a, b, c) ((J[ID(i + (a), j + (b), k + (c))] * ma[ID(i + (a), j + (b), k + (c))]) * mb[ID(i + (a), j + (b), k + (c))])
    double s = P3(m1, m2, 1, 0, 0) * (F(1, 1, 0) - F(1, -1, 0));
    s = s - P3(m1, m2, -1, 0, 0) * (F(-1, 1, 0) - F(-1, -1, 0));
    s = s + P3(m1, m3, 1, 0, 0) * (F(1, 0, 1) - F(1, 0, -1));
    s = s - P3(m1, m3, -1, 0, 0) * (F(-1, 0, 1) - F(-1, 0, -1));
    s = s + P3(m2, m1, 0, 1, 0) * (F(1, 1, 0) - F(-1, 1, 0));
    s = s - P3(m2, m1, 0, -1, 0) * (F(1, -1, 0) - F(-1, -1, 0));
    s = s + P3(m2, m3, 0, 1, 0) * (F(0, 1, 1) - F(0, 1, -1));
    s = s - P3(m2, m3, 0, -1, 0) * (F(0, -1, 1) - F(0, -1, -1));
    s = s + P3(m3, m1, 0, 0, 1) * (F(1, 0, 1) - F(-1, 0, 1));
    s = s - P3(m3, m1, 0, 0, -1) * (F(1, 0, -1) - F(-1, 0, -1));
    s = s + P3(m3, m2, 0, 0, 1) * (F(0, 1, 1) - F(0, -1, 1));
    s = s - P3(m3, m2, 0, 0, -1) * (F(0, 1, -1) - F(0, -1, -1));
#undef F
#undef P3
    return 0.25 * s;
}

/* kind 0: U, 1: V or W, 2: T.  inm: field at step n; ina, inb: NL and NL_nm1;
 * inc: DIF; ind: pressure source (NULL for T). */
static void predictor(o3 *o, int kind, double *in, const double *inm, const double *ina, const double *inb,
                      const double *inc, const double *ind)
{
    const double rek = kind == 2 ? o->pe : o->p.re;
    const int cyc = o->p.order == O3_GPU;
    for (int split = 0; split < 3; split++) {
        af_coef(o, split, rek);
        for (int k = 1; k <= o->NK - 1; k++)
            for (int j = 1; j <= o->NJ - 1; j++)
                for (int i = 1; i <= o->NI - 1; i++) o->DD[ID(i, j, k)] = af_cross(o, split, in, i, j, k);
        for (int k = 1; k <= o->NK - 1; k++)
            for (int j = 1; j <= o->NJ - 1; j++)
                for (int i = 1; i <= o->NI - 1; i++) {
                    int c = ID(i, j, k);
                    double r = ((2.0 * rek) * o->DJAC[c]) / o->p.dt;
                    if (split == 0) {
                        double s = (r * inm[c] - (3.0 * rek) * ina[c]) + (1.0 * rek) * inb[c];
                        s = s + inc[c];
                        if (ind) s = s + (2.0 * rek) * ind[c];
                        o->SU[c] = s + o->DD[c];
                    } else {
                        o->SU[c] = r * in[c] + o->DD[c];
                    }
                }
        bc_field(o, kind, in, inm);
        sweep(o, split, in, cyc);
    }
}

/* ------------------------------------------------------------------------- */
/* ITER_P (iter_p.f90:12-63) with BCP and LISOLV                              */
/* ------------------------------------------------------------------------- */
static double residual(o3 *o)
{
    const int gpu = o->p.order == O3_GPU;
    double resip = 0.0, dum = 0.0;
    const double *P = o->P;
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) {
                int c = ID(i, j, k);
                int jn = gpu ? jw(o, j + 1) : j + 1, js = gpu ? jw(o, j - 1) : j - 1;
                int kt = gpu ? kw(o, k + 1) : k + 1, kb = gpu ? kw(o, k - 1) : k - 1;
                double r = ((((((o->AE[c] * P[ID(i + 1, j, k)] + o->AW[c] * P[ID(i - 1, j, k)]) + o->AN[c] * P[ID(i, jn, k)]) +
                                o->AS[c] * P[ID(i, js, k)]) + o->AT[c] * P[ID(i, j, kt)]) + o->AB[c] * P[ID(i, j, kb)]) +
                             o->SU[c]) - o->AP[c] * P[c];
                resip = resip + fabs(r);
                dum = dum + fabs(o->AP[c] * P[c]);
            }
    return resip / dum;
}

static int iter_p(o3 *o)
{
    const int n = o->n;
    for (int c = 0; c < n; c++) {
        o->AP[c] = (((((-o->DE[c]) - o->DW[c]) - o->DN[c]) - o->DS[c]) - o->DT[c]) - o->DB[c];
        o->AE[c] = -o->DE[c];
        o->AW[c] = -o->DW[c];
        o->AN[c] = -o->DN[c];
        o->AS[c] = -o->DS[c];
        o->AT[c] = -o->DT[c];
        o->AB[c] = -o->DB[c];
    }
    const double rdt = 1.0 / o->p.dt;
    int niter = 0;
    double resip = 0.0;
    for (;;) {
        niter = niter + 1;
        dif_diagonal(o, o->P, o->DD);
        for (int k = 1; k <= o->NK - 1; k++)
            for (int j = 1; j <= o->NJ - 1; j++)
                for (int i = 1; i <= o->NI - 1; i++) {
                    int c = ID(i, j, k);
                    o->SU[c] = rdt * (((((o->UE[c] - o->UW[c]) + o->VN[c]) - o->VS[c]) + o->WT[c]) - o->WB[c]) - o->DD[c];
                }
        bcp(o);
        sweep(o, 0, o->P, 0);
        int check = (o->p.order == O3_FAITHFUL) || (niter % o->p.res_every == 0) || (niter >= o->p.nswpp);
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
/* Dynamic Smagorinsky model (stress_tensor_dy.f90, test_filter.f90)          */
/* ------------------------------------------------------------------------- */
/* TEST_FILTER (test_filter.f90:13-21): [1,2,1]^3/64 over the 27 neighbours */
void o3_test_filter(o3 *o, const double *in, double *out)
{
    static const double w[3] = {1.0, 2.0, 1.0};
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) {
                double s = 0.0;
                int first = 1;
                for (int c = -1; c <= 1; c++)
                    for (int b = -1; b <= 1; b++)
                        for (int a = -1; a <= 1; a++) {
                            double wt = (w[a + 1] * w[b + 1]) * w[c + 1];
                            double v = in[ID(i + a, j + b, k + c)];
                            double term = wt == 1.0 ? v : wt * v;
                            s = first ? term : s + term;
                            first = 0;
                        }
                out[ID(i, j, k)] = s / 64.0;
            }
}

/* xi-derivative part of a strain-rate term: m * (f(i+1) - f(i-1)) inside,
 * (2 m) * (f(1) - f(0)) on the wall ghost plane and (2 m) * (f(NI) - f(NI-1)) on
 * the far ghost plane (stress_tensor_dy.f90:96-196). */
static double dxi(const o3 *o, const double *m, const double *f, int i, int j, int k)
{
    int c = ID(i, j, k);
    if (i == 0) return (2.0 * m[c]) * (f[ID(1, j, k)] - f[c]);
    if (i == o->NI) return (2.0 * m[c]) * (f[c] - f[ID(o->NI - 1, j, k)]);
    return m[c] * (f[ID(i + 1, j, k)] - f[ID(i - 1, j, k)]);
}
static double deta(const o3 *o, const double *m, const double *f, int i, int j, int k)
{
    return m[ID(i, j, k)] * (f[ID(i, j + 1, k)] - f[ID(i, j - 1, k)]);
}
static double dzeta(const o3 *o, const double *m, const double *f, int i, int j, int k)
{
    return m[ID(i, j, k)] * (f[ID(i, j, k + 1)] - f[ID(i, j, k - 1)]);
}

/* Strain-rate components of (u, v, w) and the temperature gradient at (i,j,k):
 * S[0..8] = S11 S12 S13 S21 S22 S23 S31 S32 S33, G[0..2] = dT/dx, dT/dy, dT/dz. */
static void strain(const o3 *o, const double *u, const double *v, const double *w, const double *t, int i, int j, int k,
                   double *S, double *G)
{
    const double *M1[3] = {o->XIX, o->XIY, o->XIZ}, *M2[3] = {o->ETX, o->ETY, o->ETZ}, *M3[3] = {o->ZTX, o->ZTY, o->ZTZ};
    const double *F[3] = {u, v, w};
    /* d f / d x_dir (without the 1/2 of the centred differences) */
#define D(f, dir) ((dxi(o, M1[dir], f, i, j, k) + deta(o, M2[dir], f, i, j, k)) + dzeta(o, M3[dir], f, i, j, k))
    for (int a = 0; a < 3; a++)
        for (int b = a; b < 3; b++) {
            double val;
            if (a == b) val = 0.5 * D(F[a], a);
            else {
                /* (dx_b of u_a) + (dx_a of u_b), each as the three index-direction terms */
                double s = dxi(o, M1[b], F[a], i, j, k);
                s = s + deta(o, M2[b], F[a], i, j, k);
                s = s + dzeta(o, M3[b], F[a], i, j, k);
                s = s + dxi(o, M1[a], F[b], i, j, k);
                s = s + deta(o, M2[a], F[b], i, j, k);
                s = s + dzeta(o, M3[a], F[b], i, j, k);
                val = 0.25 * s;
            }
            S[3 * a + b] = val;
            S[3 * b + a] = val;
        }
    if (t)
        for (int d = 0; d < 3; d++) G[d] = 0.5 * D(t, d);
#undef D
}

static double sq9(const double *S)
{
    double s = S[0] * S[0];
    for (int q = 1; q < 9; q++) s = s + S[q] * S[q];
    return s;
}

/* Least-squares coefficient over the positive points of the volume
 * (stress_tensor_dy.f90:486-517), or per (i,j) along k (les_zavg). */
static double dyn_coeff(o3 *o, double *cz)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    if (!o->p.les_zavg) {
        double lm = 0.0, mm = 0.0, inc = 0.0;
        for (int k = 1; k <= NK - 1; k++)
            for (int j = 1; j <= NJ - 1; j++)
                for (int i = 1; i <= NI - 1; i++) {
                    int c = ID(i, j, k);
                    double cs = (0.5 * o->LM[c]) / o->MM[c];
                    if (cs >= 0.0) {
                        lm = lm + o->LM[c];
                        mm = mm + o->MM[c];
                        inc = inc + 1.0;
                    }
                }
        lm = lm / inc;
        mm = mm / inc;
        double cavg = (0.5 * lm) / mm;
        if (mm < 1e-6) cavg = 0.0;
        return cavg;
    }
    for (int j = 1; j <= NJ - 1; j++)
        for (int i = 1; i <= NI - 1; i++) {
            double lm = 0.0, mm = 0.0;
            for (int k = 1; k <= NK - 1; k++) {
                lm = lm + o->LM[ID(i, j, k)];
                mm = mm + o->MM[ID(i, j, k)];
            }
            double cc = mm > 0.0 ? (0.5 * lm) / mm : 0.0;
            cz[i + (NI + 1) * j] = cc > 0.0 ? cc : 0.0;
        }
    return 0.0;
}

/* Eddy coefficient field: C * FW^2 * |S| over the whole array (the z-averaged
 * coefficient of the nearest interior column at the ghost cells). */
static void eddy_field(o3 *o, double cavg, const double *cz, double *out)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    for (int k = 0; k <= NK; k++)
        for (int j = 0; j <= NJ; j++)
            for (int i = 0; i <= NI; i++) {
                int c = ID(i, j, k);
                double cc = cavg;
                if (o->p.les_zavg) {
                    int ii = i < 1 ? 1 : (i > NI - 1 ? NI - 1 : i);
                    cc = cz[ii + (NI + 1) * jw(o, j)];
                }
                out[c] = (cc * (o->FW[c] * o->FW[c])) * o->MAG[c];
            }
}

/* SGS divergence term: 0.5 sum_dir sum_index m * (-2 E L (+1) + 2 E L (-1)) */
static double sgs_div(const o3 *o, const double *E, const double *const *Lc, int i, int j, int k)
{
    const double *M1[3] = {o->XIX, o->XIY, o->XIZ}, *M2[3] = {o->ETX, o->ETY, o->ETZ}, *M3[3] = {o->ZTX, o->ZTY, o->ZTZ};
    int c = ID(i, j, k);
    double s = 0.0;
    int first = 1;
    for (int b = 0; b < 3; b++) {
        const double *L = Lc[b];
        int ip = ID(i + 1, j, k), im = ID(i - 1, j, k), jp = ID(i, j + 1, k), jm = ID(i, j - 1, k), kp = ID(i, j, k + 1),
            km = ID(i, j, k - 1);
        double t1 = M1[b][c] * (-((2.0 * E[ip]) * L[ip]) + (2.0 * E[im]) * L[im]);
        double t2 = M2[b][c] * (-((2.0 * E[jp]) * L[jp]) + (2.0 * E[jm]) * L[jm]);
        double t3 = M3[b][c] * (-((2.0 * E[kp]) * L[kp]) + (2.0 * E[km]) * L[km]);
        s = first ? t1 : s + t1;
        first = 0;
        s = s + t2;
        s = s + t3;
    }
    return 0.5 * s;
}

/* STRESS_TENSOR_DY (stress_tensor_dy.f90:20-735): SGS_X, SGS_Y, SGS_Z, SGS_T */
void o3_sgs(o3 *o)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK, n = o->n;
    const int thermal = o->p.thermal;
    for (int c = 0; c < n; c++) o->FW[c] = pow(o->DJAC[c], 1.0 / 3.0);
    double S[9], G[3];
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 0; i <= NI; i++) {
                strain(o, o->U, o->V, o->W, o->T, i, j, k, S, G);
                for (int q = 0; q < 9; q++) o->L[q][ID(i, j, k)] = S[q];
                for (int d = 0; d < 3; d++) o->DTD[d][ID(i, j, k)] = G[d];
            }
    for (int q = 0; q < 9; q++) halo(o, o->L[q]);
    for (int d = 0; d < 3; d++) halo(o, o->DTD[d]);
    for (int c = 0; c < n; c++) {
        double s = o->L[0][c] * o->L[0][c];
        for (int q = 1; q < 9; q++) s = s + o->L[q][c] * o->L[q][c];
        o->MAG[c] = sqrt(2.0 * s);
    }
    o3_test_filter(o, o->U, o->UH);
    o3_test_filter(o, o->V, o->VH);
    o3_test_filter(o, o->W, o->WH);
    o3_test_filter(o, o->T, o->TH);
    bc_field(o, 0, o->UH, o->U_N);
    bc_field(o, 1, o->VH, o->V_N);
    bc_field(o, 1, o->WH, o->W_N);
    bc_field(o, 2, o->TH, o->T_N);
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++) {
                strain(o, o->UH, o->VH, o->WH, NULL, i, j, k, S, G);
                o->MAGH[ID(i, j, k)] = sqrt(2.0 * sq9(S));
            }
    /* Germano identity terms, components 11, 22, 33, 12, 13, 23 */
    const double *uf[3] = {o->U, o->V, o->W}, *uh[3] = {o->UH, o->VH, o->WH};
    static const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
    double *cz = (double *)calloc((size_t)(NI + 1) * (NJ + 1), sizeof(double));
    for (int q = 0; q < 6; q++) {
        const int a = pa[q], b = pb[q];
        for (int c = 0; c < n; c++) o->DIN[c] = uf[a][c] * uf[b][c];
        o3_test_filter(o, o->DIN, o->DOUT);
        for (int k = 1; k <= NK - 1; k++)
            for (int j = 1; j <= NJ - 1; j++)
                for (int i = 1; i <= NI - 1; i++) {
                    int c = ID(i, j, k);
                    o->LIJ[c] = (-o->DOUT[c]) + uh[a][c] * uh[b][c];
                }
        for (int c = 0; c < n; c++) o->DIN[c] = o->MAG[c] * o->L[3 * a + b][c];
        o3_test_filter(o, o->DIN, o->DOUT);
        for (int k = 1; k <= NK - 1; k++)
            for (int j = 1; j <= NJ - 1; j++)
                for (int i = 1; i <= NI - 1; i++) {
                    int c = ID(i, j, k);
                    strain(o, o->UH, o->VH, o->WH, NULL, i, j, k, S, G);
                    /* hat strain without its leading factor: 0.5 or 0.25 times the sum */
                    double hs;
                    if (a == b) hs = S[3 * a + b] / 0.5;
                    else hs = S[3 * a + b] / 0.25;
                    double fac = a == b ? 0.5 : 0.25;
                    double m = ((4.0 * o->MAGH[c]) * fac) * hs;
                    m = (o->FW[c] * o->FW[c]) * (m - o->DOUT[c]);
                    double l = o->LIJ[c];
                    if (q == 0) {
                        o->LM[c] = l * m;
                        o->MM[c] = m * m;
                    } else if (q < 3) {
                        o->LM[c] = o->LM[c] + l * m;
                        o->MM[c] = o->MM[c] + m * m;
                    } else {
                        o->LM[c] = o->LM[c] + (2.0 * l) * m;
                        o->MM[c] = o->MM[c] + (2.0 * m) * m;
                    }
                }
    }
    double cavg = dyn_coeff(o, cz);
    o->co.cs2 = cavg;
    eddy_field(o, cavg, cz, o->EV);
    const double *rows[3][3] = {{o->L[0], o->L[1], o->L[2]}, {o->L[3], o->L[4], o->L[5]}, {o->L[6], o->L[7], o->L[8]}};
    double *out[3] = {o->SGSX, o->SGSY, o->SGSZ};
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= NI - 1; i++)
                for (int r = 0; r < 3; r++) out[r][ID(i, j, k)] = sgs_div(o, o->EV, rows[r], i, j, k);
    if (thermal) {
        for (int q = 0; q < 3; q++) {
            for (int c = 0; c < n; c++) o->DIN[c] = uf[q][c] * o->T[c];
            o3_test_filter(o, o->DIN, o->DOUT);
            for (int k = 1; k <= NK - 1; k++)
                for (int j = 1; j <= NJ - 1; j++)
                    for (int i = 1; i <= NI - 1; i++) {
                        int c = ID(i, j, k);
                        o->LIJ[c] = (-o->DOUT[c]) + uh[q][c] * o->TH[c];
                    }
            for (int c = 0; c < n; c++) o->DIN[c] = o->MAG[c] * o->DTD[q][c];
            o3_test_filter(o, o->DIN, o->DOUT);
            const double *M1[3] = {o->XIX, o->XIY, o->XIZ}, *M2[3] = {o->ETX, o->ETY, o->ETZ},
                         *M3[3] = {o->ZTX, o->ZTY, o->ZTZ};
            for (int k = 1; k <= NK - 1; k++)
                for (int j = 1; j <= NJ - 1; j++)
                    for (int i = 1; i <= NI - 1; i++) {
                        int c = ID(i, j, k);
                        double g = (dxi(o, M1[q], o->TH, i, j, k) + deta(o, M2[q], o->TH, i, j, k)) +
                                   dzeta(o, M3[q], o->TH, i, j, k);
                        double m = ((4.0 * o->MAGH[c]) * 0.5) * g;
                        m = (o->FW[c] * o->FW[c]) * (m - o->DOUT[c]);
                        double l = o->LIJ[c];
                        if (q == 0) {
                            o->LM[c] = l * m;
                            o->MM[c] = m * m;
                        } else {
                            o->LM[c] = o->LM[c] + l * m;
                            o->MM[c] = o->MM[c] + m * m;
                        }
                    }
        }
        double ct = dyn_coeff(o, cz);
        o->co.ct2 = ct;
        eddy_field(o, ct, cz, o->EC);
        const double *gr[3] = {o->DTD[0], o->DTD[1], o->DTD[2]};
        for (int k = 1; k <= NK - 1; k++)
            for (int j = 1; j <= NJ - 1; j++)
                for (int i = 1; i <= NI - 1; i++) o->SGST[ID(i, j, k)] = sgs_div(o, o->EC, gr, i, j, k);
    }
    free(cz);
}

/* ------------------------------------------------------------------------- */
/* CALCCOEF (calccoef.f90:9-160)                                              */
/* ------------------------------------------------------------------------- */
/* The post-processing block of CALCCOEF (calccoef.f90:286-307): sums over the
 * whole array, the SGS stress as -2 nu_t S_ij of the step's model. */
static void post_sums(o3 *o)
{
    o->niter_pos = o->niter_pos + 1;
    const double *f[3] = {o->U, o->V, o->W};
    static const int ra[] = {0, 0, 0, 1, 1, 2}, rb[] = {0, 1, 2, 1, 2, 2}, ls[] = {0, 1, 2, 4, 5, 8};
    for (int c = 0; c < o->n; c++) {
        o->PS[0][c] = o->PS[0][c] + o->U[c];
        o->PS[1][c] = o->PS[1][c] + o->V[c];
        o->PS[2][c] = o->PS[2][c] + o->W[c];
        o->PS[3][c] = o->PS[3][c] + o->P[c];
        o->PS[4][c] = o->PS[4][c] + o->T[c];
        for (int q = 0; q < 6; q++) o->PS[5 + q][c] = o->PS[5 + q][c] + f[ra[q]][c] * f[rb[q]][c];
        for (int q = 0; q < 6; q++) o->PS[11 + q][c] = o->PS[11 + q][c] - (2.0 * o->EV[c]) * o->L[ls[q]][c];
    }
}

static void calccoef(o3 *o)
{
    const int NI = o->NI, NJ = o->NJ, NK = o->NK;
    (void)NI;
    double cfl = 0.0;
    for (int k = 1; k <= NK - 1; k++)
        for (int j = 1; j <= NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) {
                int c = ID(i, j, k);
                double l = o->p.dt * ((fabs((o->XIX[c] * o->U[c] + o->XIY[c] * o->V[c]) + o->XIZ[c] * o->W[c]) +
                                       fabs((o->ETX[c] * o->U[c] + o->ETY[c] * o->V[c]) + o->ETZ[c] * o->W[c])) +
                                      fabs((o->ZTX[c] * o->U[c] + o->ZTY[c] * o->V[c]) + o->ZTZ[c] * o->W[c]));
                cfl = cfl > l ? cfl : l;
            }
    const double *P = o->P;
    double dumb = 0.0;
    for (int k = 1; k <= NK - 1; k++) {
        const int i = 1, j = 1;
        double pg = 0.125 * (((((((P[ID(i, j, k)] + P[ID(i, j - 1, k)]) + P[ID(i - 1, j, k)]) + P[ID(i - 1, j - 1, k)]) +
                                P[ID(i, j, k + 1)]) + P[ID(i, j - 1, k + 1)]) + P[ID(i - 1, j, k + 1)]) +
                             P[ID(i - 1, j - 1, k + 1)]);
        dumb = dumb + pg;
    }
    dumb = dumb / (double)(NK - 1);
    double cpb = 0.0 + 2.0 * (0.0 - dumb);
    double pd = 0.0, pl = 0.0, td = 0.0, tl = 0.0, snu = 0.0;
    const double *XG = o->XG, *YG = o->YG, *ZG = o->ZG;
    for (int tri = 0; tri < 2; tri++)
        for (int k = 1; k <= NK - 1; k++)
            for (int j = 1; j <= NJ - 1; j++) {
                const int i = 1, c = ID(i, j, k);
                int p, q, r;
                if (tri == 0) { p = ID(i, j, k); q = ID(i, j + 1, k); r = ID(i, j, k + 1); }
                else { p = ID(i, j + 1, k + 1); q = ID(i, j, k + 1); r = ID(i, j, k); }
                double A = (YG[p] * (ZG[q] - ZG[r]) + YG[q] * (ZG[r] - ZG[p])) + YG[r] * (ZG[p] - ZG[q]);
                double B = (ZG[p] * (XG[q] - XG[r]) + ZG[q] * (XG[r] - XG[p])) + ZG[r] * (XG[p] - XG[q]);
                double C = (XG[p] * (YG[q] - YG[r]) + XG[q] * (YG[r] - YG[p])) + XG[r] * (YG[p] - YG[q]);
                double D = (XG[p] * (YG[q] * ZG[r] - YG[r] * ZG[q]) + XG[q] * (YG[r] * ZG[p] - YG[p] * ZG[r])) +
                           XG[r] * (YG[p] * ZG[q] - YG[q] * ZG[p]);
                D = -1.0 * D;
                double dum = sqrt((A * A + B * B) + C * C);
                double dn = fabs(((A * o->X[c] + B * o->Y[c]) + C * o->Z[c]) + D) / dum;
                double u = o->U[c], v = o->V[c], w = o->W[c];
                double e1 = (v * C) / dum - (w * B) / dum, e2 = (u * C) / dum - (w * A) / dum, e3 = (u * B) / dum - (v * A) / dum;
                double dudn = sqrt((e1 * e1 + e2 * e2) + e3 * e3);
                dudn = dudn / dn;
                double area = tri == 0 ? o->AREA1[c] : o->AREA2[c];
                double vm = sqrt((u * u + v * v) + w * w);
                pd = pd - (((2.0 * P[c]) * area) * A) / dum;
                pl = pl - (((2.0 * P[c]) * area) * B) / dum;
                td = td + ((((2.0 / o->p.re) * dudn) * area) * u) / vm;
                tl = tl + ((((2.0 / o->p.re) * dudn) * area) * v) / vm;
                double dtdn = (o->T[c] - o->p.t_wall) / dn;
                snu = snu + dtdn * area;
            }
    o3_coeffs *co = &o->co;
    co->time = o->rtime;
    co->cfl = cfl;
    co->cpb = cpb;
    co->cd_p = pd / o->p.ref_a;
    co->cl_p = pl / o->p.ref_a;
    co->cd_v = td / o->p.ref_a;
    co->cl_v = tl / o->p.ref_a;
    co->cd = co->cd_p + co->cd_v;
    co->cl = co->cl_p + co->cl_v;
    co->nu = -snu / o->sum_area;
    if (o->ipost) post_sums(o);
}

/* ------------------------------------------------------------------------- */
/* Post-processing (post_process.f90:8-285, calccoef.f90:286-307)              */
/* ------------------------------------------------------------------------- */
void o3_post_begin(o3 *o)
{
    for (int q = 0; q < 17; q++) memset(o->PS[q], 0, sizeof(double) * (size_t)o->n);
    o->niter_pos = 0;
    o->ipost = 1;
}

int o3_post_steps(const o3 *o) { return o->niter_pos; }

/* The wall statistics of the averaged fields at the wall cell (1, j, k): shear
 * rate, wall heat flux and the pressure of the wall node, over the face's two
 * triangles (post_process.f90:67-116), scaled as written out (:252-255). */
static void wall_stats(const o3 *o, const double *ua, const double *va, const double *wa, const double *pa,
                       const double *ta, int j, int k, double *cf, double *cp, double *nu)
{
    const double *XG = o->XG, *YG = o->YG, *ZG = o->ZG;
    const int i = 1, c = ID(i, j, k);
    double sh = 0.0, nus = 0.0;
    for (int tri = 0; tri < 2; tri++) {
        int p, q, r;
        if (tri == 0) { p = ID(i, j, k); q = ID(i, j + 1, k); r = ID(i, j, k + 1); }
        else { p = ID(i, j + 1, k + 1); q = ID(i, j, k + 1); r = ID(i, j, k); }
        double A = (YG[p] * (ZG[q] - ZG[r]) + YG[q] * (ZG[r] - ZG[p])) + YG[r] * (ZG[p] - ZG[q]);
        double B = (ZG[p] * (XG[q] - XG[r]) + ZG[q] * (XG[r] - XG[p])) + ZG[r] * (XG[p] - XG[q]);
        double C = (XG[p] * (YG[q] - YG[r]) + XG[q] * (YG[r] - YG[p])) + XG[r] * (YG[p] - YG[q]);
        double D = (XG[p] * (YG[q] * ZG[r] - YG[r] * ZG[q]) + XG[q] * (YG[r] * ZG[p] - YG[p] * ZG[r])) +
                   XG[r] * (YG[p] * ZG[q] - YG[q] * ZG[p]);
        D = -1.0 * D;
        double dum = sqrt((A * A + B * B) + C * C);
        double dn = fabs(((A * o->X[c] + B * o->Y[c]) + C * o->Z[c]) + D) / dum;
        double u = ua[c], v = va[c], w = wa[c];
        double e1 = (v * C) / dum - (w * B) / dum, e2 = (u * C) / dum - (w * A) / dum, e3 = (u * B) / dum - (v * A) / dum;
        double dudn = sqrt((e1 * e1 + e2 * e2) + e3 * e3);
        dudn = dudn / dn;
        double dtdn = (ta[c] - o->p.t_wall) / dn;
        double ar = tri == 0 ? o->AREA1[c] : o->AREA2[c];
        double tot = o->AREA1[c] + o->AREA2[c];
        sh = sh + (dudn * ar) / tot;
        nus = nus + (dtdn * ar) / tot;
    }
    double pg = 0.125 * (((((((pa[ID(i, j, k)] + pa[ID(i, j - 1, k)]) + pa[ID(i - 1, j, k)]) + pa[ID(i - 1, j - 1, k)]) +
                            pa[ID(i, j, k + 1)]) + pa[ID(i, j - 1, k + 1)]) + pa[ID(i - 1, j, k + 1)]) +
                         pa[ID(i - 1, j - 1, k + 1)]);
    *cf = (2.0 / sqrt(o->p.re)) * sh;
    *cp = 2.0 * pg;
    *nu = -nus;
}

/* POST_PROCESS with IPOST=1: "U_AVG".."T_AVG", the Reynolds stresses with their SGS
 * part "UU","UV","UW","VV","VW","WW" (post_process.f90:207-212), "U_RMS".."W_RMS"
 * (the root mean squares, :164-166), full arrays; "CF_WALL","CP_WALL","NU_WALL" at
 * out[j + (NJ+1) k] for the wall cells.  Returns -1 for an unknown name or before
 * any averaged step. */
int o3_post_get(o3 *o, const char *name, double *out)
{
    const int n = o->n;
    if (o->niter_pos < 1) return -1;
    const double N = (double)o->niter_pos;
    static const char *avg[] = {"U_AVG", "V_AVG", "W_AVG", "P_AVG", "T_AVG"};
    for (int q = 0; q < 5; q++)
        if (!strcmp(name, avg[q])) {
            for (int c = 0; c < n; c++) out[c] = o->PS[q][c] / N;
            return 0;
        }
    static const char *rs[] = {"UU", "UV", "UW", "VV", "VW", "WW"};
    static const int ra[] = {0, 0, 0, 1, 1, 2}, rb[] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; q++)
        if (!strcmp(name, rs[q])) {
            for (int c = 0; c < n; c++) {
                double m = o->PS[5 + q][c] / N, a = o->PS[ra[q]][c] / N, b = o->PS[rb[q]][c] / N;
                out[c] = (m - a * b) + o->PS[11 + q][c] / N;
            }
            return 0;
        }
    static const char *rms[] = {"U_RMS", "V_RMS", "W_RMS"};
    static const int rq[] = {5, 8, 10};
    for (int q = 0; q < 3; q++)
        if (!strcmp(name, rms[q])) {
            for (int c = 0; c < n; c++) out[c] = sqrt(o->PS[rq[q]][c] / N);
            return 0;
        }
    int which = !strcmp(name, "CF_WALL") ? 0 : (!strcmp(name, "CP_WALL") ? 1 : (!strcmp(name, "NU_WALL") ? 2 : -1));
    if (which < 0) return -1;
    double *a[5];
    for (int q = 0; q < 5; q++) {
        a[q] = (double *)malloc(sizeof(double) * (size_t)n);
        for (int c = 0; c < n; c++) a[q][c] = o->PS[q][c] / N;
    }
    for (int c = 0; c < o->NJ1 * (o->NK + 1); c++) out[c] = 0.0;
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++) {
            double v[3];
            wall_stats(o, a[0], a[1], a[2], a[3], a[4], j, k, &v[0], &v[1], &v[2]);
            out[j + o->NJ1 * k] = v[which];
        }
    for (int q = 0; q < 5; q++) free(a[q]);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Time step (main.f90:33-147)                                                 */
/* ------------------------------------------------------------------------- */
static void add_dt_s(o3 *o, double sign)
{
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) {
                int c = ID(i, j, k);
                double f = o->p.dt;
                if (sign < 0) {
                    o->U[c] = o->U[c] - (f * o->S_U[c]) / o->DJAC[c];
                    o->V[c] = o->V[c] - (f * o->S_V[c]) / o->DJAC[c];
                    o->W[c] = o->W[c] - (f * o->S_W[c]) / o->DJAC[c];
                } else {
                    o->U[c] = o->U[c] + (f * o->S_U[c]) / o->DJAC[c];
                    o->V[c] = o->V[c] + (f * o->S_V[c]) / o->DJAC[c];
                    o->W[c] = o->W[c] + (f * o->S_W[c]) / o->DJAC[c];
                }
            }
}

static void copy_int(o3 *o, const double *src, double *dst)
{
    for (int k = 1; k <= o->NK - 1; k++)
        for (int j = 1; j <= o->NJ - 1; j++)
            for (int i = 1; i <= o->NI - 1; i++) dst[ID(i, j, k)] = src[ID(i, j, k)];
}

int o3_step(o3 *o, int nsteps)
{
    const int n = o->n;
    for (int s = 0; s < nsteps; s++) {
        o->niter_time = o->niter_time + 1;
        o->rtime = o->rtime + o->p.dt;
        memcpy(o->U_N, o->U, sizeof(double) * (size_t)n);
        memcpy(o->V_N, o->V, sizeof(double) * (size_t)n);
        memcpy(o->W_N, o->W, sizeof(double) * (size_t)n);
        memcpy(o->T_N, o->T, sizeof(double) * (size_t)n);
        contra_vel(o);
        copy_int(o, o->NLX, o->NLX_NM1);
        copy_int(o, o->NLY, o->NLY_NM1);
        copy_int(o, o->NLZ, o->NLZ_NM1);
        copy_int(o, o->ADV, o->ADV_NM1);
        nl(o, o->U_N, o->NLX);
        nl(o, o->V_N, o->NLY);
        nl(o, o->W_N, o->NLZ);
        if (o->p.thermal) nl(o, o->T_N, o->ADV);
        if (o->p.use_les) {
            o3_sgs(o);
            for (int k = 1; k <= o->NK - 1; k++)
                for (int j = 1; j <= o->NJ - 1; j++)
                    for (int i = 1; i <= o->NI - 1; i++) {
                        int c = ID(i, j, k);
                        o->NLX[c] = o->NLX[c] + o->SGSX[c] * o->DJAC[c];
                        o->NLY[c] = o->NLY[c] + o->SGSY[c] * o->DJAC[c];
                        o->NLZ[c] = o->NLZ[c] + o->SGSZ[c] * o->DJAC[c];
                        if (o->p.thermal) o->ADV[c] = o->ADV[c] + o->SGST[c] * o->DJAC[c];
                    }
        }
        dif(o, o->U_N, o->DIFX);
        dif(o, o->V_N, o->DIFY);
        dif(o, o->W_N, o->DIFZ);
        if (o->p.thermal) dif(o, o->T_N, o->DIFT);
        p_source(o, o->P);
        predictor(o, 0, o->U, o->U_N, o->NLX, o->NLX_NM1, o->DIFX, o->S_U);
        predictor(o, 1, o->V, o->V_N, o->NLY, o->NLY_NM1, o->DIFY, o->S_V);
        predictor(o, 1, o->W, o->W_N, o->NLZ, o->NLZ_NM1, o->DIFZ, o->S_W);
        add_dt_s(o, -1.0);
        bc_field(o, 0, o->U, o->U_N);
        bc_field(o, 1, o->V, o->V_N);
        bc_field(o, 1, o->W, o->W_N);
        contra_vel(o);
        iter_p(o);
        bcp(o);
        p_source(o, o->P);
        add_dt_s(o, +1.0);
        /* reference pressure at the far-field node column (I = NI, J = NJ/4) */
        double dumb = 0.0;
        for (int k = 1; k <= o->NK - 1; k++) dumb = dumb + o->P[ID(o->NI, o->NJ / 4, k)];
        dumb = dumb / (double)(o->NK - 1);
        for (int c = 0; c < n; c++) o->P[c] = o->P[c] - dumb;
        bc_field(o, 0, o->U, o->U_N);
        bc_field(o, 1, o->V, o->V_N);
        bc_field(o, 1, o->W, o->W_N);
        if (o->p.thermal) {
            predictor(o, 2, o->T, o->T_N, o->ADV, o->ADV_NM1, o->DIFT, NULL);
            bc_field(o, 2, o->T, o->T_N);
        }
        calccoef(o);
        for (int c = 0; c < n; c++)
            if (!isfinite(o->U[c]) || !isfinite(o->P[c])) return -1;
    }
    return 0;
}

double *o3_array(o3 *o, const char *name)
{
    struct { const char *n; double *a; } t[] = {
        {"U", o->U}, {"V", o->V}, {"W", o->W}, {"P", o->P}, {"T", o->T}, {"NLX", o->NLX}, {"NLY", o->NLY},
        {"NLZ", o->NLZ}, {"ADV", o->ADV}, {"X", o->X}, {"Y", o->Y}, {"Z", o->Z}, {"DJAC", o->DJAC},
        {"XIX", o->XIX}, {"XIY", o->XIY}, {"XIZ", o->XIZ}, {"ETX", o->ETX}, {"ETY", o->ETY}, {"ETZ", o->ETZ},
        {"ZTX", o->ZTX}, {"ZTY", o->ZTY}, {"ZTZ", o->ZTZ}, {"DE", o->DE}, {"DN", o->DN}, {"DT", o->DT},
        {"THETA", o->THETA}, {"SGS_X", o->SGSX}, {"SGS_Y", o->SGSY}, {"SGS_Z", o->SGSZ}, {"SGS_T", o->SGST},
        {"EDDY_VISCOS", o->EV}, {"MAG", o->MAG}, {"U_HAT", o->UH}, {"DIFX", o->DIFX}, {"S_U", o->S_U},
        {"UE", o->UE}, {"VN", o->VN}, {"WT", o->WT}, {"XG", o->XG}, {"YG", o->YG}, {"ZG", o->ZG},
        {"U_N", o->U_N}, {"V_N", o->V_N}, {"W_N", o->W_N}, {"T_N", o->T_N}, {"NLX_NM1", o->NLX_NM1},
        {"NLY_NM1", o->NLY_NM1}, {"NLZ_NM1", o->NLZ_NM1}, {"ADV_NM1", o->ADV_NM1}};
    for (size_t q = 0; q < sizeof(t) / sizeof(t[0]); q++)
        if (!strcmp(t[q].n, name)) return t[q].a;
    return NULL;
}
