// fvm_adjoint.cu -- hand-written discrete adjoint of the time step (GPU order,
// FP64): gradient of the drag coefficient averaged over a window of steps with
// respect to the wall rotation rate and the wall-normal blowing speeds.
//
// The step maps S^n = (U, V, P with their ghost cells, NLX, NLY) to S^{n+1}; the
// passive temperature does not act on them and is left out.  Taking the Poisson
// iteration as converged, the map is quadratic: every sub-step is linear in the
// state and the controls except the advection term NL, which is bilinear in the
// field and the face fluxes (nl.f90:21-27).  The adjoint runs the sub-steps in
// reverse, each transposed exactly as the forward code executes it:
//   - the Dirichlet ghost maps of BCU/BCV (wall, far field, branch cut, corners)
//     and the BCP ghost map fold the ghost adjoints back onto the interior;
//   - zebra line sweeps are reversed colour by colour: the line solve transposed
//     (factors of the transposed line matrices, cyclic ones by Sherman-Morrison),
//     the couplings to the other colour scattered with the forward coefficients;
//   - the converged Poisson equation (A + DD G) P = DIV/dt (A with the BCP folding,
//     DD the lagged cross term paired by position, G the BCP ghost map) is solved
//     transposed, (A^T + G^T DD^T) mu = g, by the same zebra line Gauss-Seidel with
//     the transposed cross term lagged;
//   - stencil operators (fluxes, NL, DIF, cross terms, P_SOURCE, the far-field
//     formula) are transposed by scattering with atomic adds.
// Checkpoints of the state are kept every `ckpt` steps of the forward pass; each
// segment is recomputed from its checkpoint (storing U and V before every step,
// the base point of NL) and then reversed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fvm_internal.cuh"
#include "fvm_ops.cuh"
#include "fvm_df.cuh"

namespace fvm {

// Adjoint arrays (device) and the transposed line systems.
struct Adj {
    double *lU, *lV, *lP, *lNLX, *lNLY;     // adjoint of the state after the step being reversed
    double *lUn, *lVn;                       // accumulators of the adjoint of U^n, V^n (full arrays)
    double *lW, *lWV;                        // interior scratch (ghost-map transposes)
    double *lSc, *lScV, *lSe, *lSeV;         // S_U/S_V adjoints of the correction and of the explicit phase
    double *lPf, *g, *mu, *XD;               // Poisson adjoint: source, solution, lagged cross term
    double *lUh, *lVh;                       // adjoint of u-hat, v-hat (full arrays)
    double *lSU, *lSUV;                      // predictor right-hand side adjoints
    double *lFE, *lFW, *lFN, *lFS;           // face flux adjoints (UE, UW, VN, VS)
    double *lUFW, *lVFW, *lFFU, *lFFV;       // wall / far-field value adjoints per j
    double *lblow;                           // blowing adjoint through the wall face flux, per j
    double *lomega;                          // [0]: rotation adjoint through the drag formula
    double *DCU, *DCV, *DCP;                 // dCd/dU(1,j), dCd/dV(1,j), dCd/dP(1,j)
    double *DCW;                             // [0]: dCd/d(omega) through the drag formula
    Coef cPT, cXT, cYT;                      // transposed coefficient sets (Poisson, first, second factor)
    LineSys sPT, sXT, sYT;                   // their line factors
    PCtl *pctl;                              // adjoint Poisson iteration control
    double *partial;
};

namespace {

// ---------------------------------------------------------------------------------
// Geometry of the drag formula (calccoef.f90:50-98 as in k_calc_rows): wall-normal
// distance DN1 and normal angle TH2 of the first cell of column j.
// ---------------------------------------------------------------------------------
__device__ void wall_normal(const Dev &d, int j, double &DN1, double &TH2)
{
    const int c = IDX(1, j);
    const double X = d.X[c], Y = d.Y[c];
    const double xa = d.XG[IDX(1, j)], ya = d.YG[IDX(1, j)], xb = d.XG[IDX(1, j + 1)], yb = d.YG[IDX(1, j + 1)];
    double L1 = ::sqrt((X - xa) * (X - xa) + (Y - ya) * (Y - ya));
    double L2 = ::sqrt((X - xb) * (X - xb) + (Y - yb) * (Y - yb));
    double L3 = ::sqrt((xb - xa) * (xb - xa) + (yb - ya) * (yb - ya));
    double TH1 = acos((((L1 * L1) + (L2 * L2)) - (L3 * L3)) / ((2.0 * L1) * L2));
    DN1 = ((L1 * L2) / L3) * sin(TH1);
    double LA = (yb - ya) / (xb - xa);
    double LB = ya - LA * xa;
    double LA_ = -1.0 / LA;
    double LB_ = Y - LA_ * X;
    double X1 = (LB_ - LB) / (LA - LA_);
    double Y1 = (LA * (LB_ - LB)) / (LA - LA_) + LB;
    double DN2 = ::sqrt((Y - Y1) * (Y - Y1) + (X - X1) * (X - X1));
    TH2 = atan((Y - Y1) / (X - X1));
    double sg = asin((Y - Y1) / DN2);
    if (TH2 >= 0.0 && sg > 0.0) TH2 = TH2;
    else if (TH2 < 0.0 && sg > 0.0) TH2 = d.pi + TH2;
    else if (TH2 >= 0.0 && sg <= 0.0) TH2 = d.pi + TH2;
    else if (TH2 < 0.0 && sg < 0.0) TH2 = 2.0 * d.pi + TH2;
}

// Cd = sum_j [-2 P(1,j) A cos th + (2/Re) A sin th ((U sin TH2 - V cos TH2) - omega)/DN1]
__global__ void k_adj_dragcoef(Dev d, Adj a)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > d.NJ - 1) return;
    double DN1, TH2;
    wall_normal(d, j, DN1, TH2);
    const int c = IDX(1, j);
    const double th = d.THETA[c], ar = d.AREA[c];
    const double v = ((2.0 / d.re) * ar) * sin(th) / DN1;
    a.DCP[j] = -((2.0 * ar) * cos(th));
    a.DCU[j] = v * sin(TH2);
    a.DCV[j] = -v * cos(TH2);
    atomicAdd(a.DCW, -v);
}

// Transposed five-point set: AE'(i,j) = AW(i+1,j), AW'(i,j) = AE(i-1,j),
// AN'(i,j) = AS(i,j+1), AS'(i,j) = AN(i,j-1) (periodic in j), AP' = AP.
__global__ void k_adj_coef_t(Dev d, Coef src, Coef dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    dst.AP[c] = src.AP[c];
    dst.AE[c] = (i < d.NI - 1) ? src.AW[IDX(i + 1, j)] : 0.0;
    dst.AW[c] = (i > 1) ? src.AE[IDX(i - 1, j)] : 0.0;
    dst.AN[c] = src.AS[IDX(i, jwrap(d, j + 1))];
    dst.AS[c] = src.AN[IDX(i, jwrap(d, j - 1))];
}

// ---------------------------------------------------------------------------------
// Ghost maps transposed
// ---------------------------------------------------------------------------------
// Dirichlet ghost map of BCU/BCV as ghost_dirichlet writes it from the interior
// values w: phi(0,j) = -w(1,j) + 2 wallF(j), phi(NI,j) = -w(NI-1,j) + 2 farF(j),
// phi(i,0) = w(i,NJ-1), phi(i,NJ) = w(i,1), corners from the cells (1|NI-1, 1|NJ-1).
// Folds the adjoint of the whole array lphi into the interior adjoint out (added),
// the wall / far-field value adjoints, and clears lphi's ghosts.
__global__ void k_adj_gd(Dev d, double *lphi, double *out, double *lwall, double *lfar, int overwrite)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    const int NI = d.NI, NJ = d.NJ;
    if (i > NI - 1 || j > NJ - 1) return;
    double s = lphi[IDX(i, j)];
    if (j == 1) s += lphi[IDX(i, NJ)];
    if (j == NJ - 1) s += lphi[IDX(i, 0)];
    if (i == 1) {
        double g = lphi[IDX(0, j)];
        if (j == 1) g += lphi[IDX(0, NJ)];
        if (j == NJ - 1) g += lphi[IDX(0, 0)];
        s -= g;
        lwall[j] += 2.0 * g;
    }
    if (i == NI - 1) {
        double g = lphi[IDX(NI, j)];
        if (j == 1) g += lphi[IDX(NI, NJ)];
        if (j == NJ - 1) g += lphi[IDX(NI, 0)];
        s -= g;
        lfar[j] += 2.0 * g;
    }
    out[IDX(i, j)] = overwrite ? s : out[IDX(i, j)] + s;
}

// Clear the ghost cells of a full array (after their adjoint has been folded).
__global__ void k_adj_clear_ghosts(Dev d, double *a)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int NI = d.NI, NJ = d.NJ;
    if (t <= NJ) {
        a[IDX(0, t)] = 0.0;
        a[IDX(NI, t)] = 0.0;
    }
    if (t <= NI) {
        a[IDX(t, 0)] = 0.0;
        a[IDX(t, NJ)] = 0.0;
    }
}

// BCP ghost map G (bcp.f90:19-42 as k_bcp_ghosts writes it) transposed: interior
// adjoint of a full-array adjoint L.
__device__ __forceinline__ double gfull_t(const Dev &d, const double *L, int i, int j)
{
    const int NI = d.NI, NJ = d.NJ;
    double s = L[IDX(i, j)];
    if (j == NJ - 1) s += L[IDX(i, 0)];
    if (j == 1) s += L[IDX(i, NJ)];
    if (i == 1) {
        s += L[IDX(0, j)];
        if (j == NJ - 1) s += L[IDX(0, 0)];
        if (j == 1) s += L[IDX(0, NJ)];
    }
    double w = 0.0;
    if (i == NI - 1) w += 3.0;
    if (i == NI - 2) w -= 3.0;
    if (i == NI - 3) w += 1.0;
    if (w != 0.0) {
        double gsum = L[IDX(NI, j)];
        if (j == NJ - 1) gsum += L[IDX(NI, 0)];
        if (j == 1) gsum += L[IDX(NI, NJ)];
        s += w * gsum;
    }
    return s;
}

__global__ void k_adj_gfull(Dev d, const double *L, double *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    out[IDX(i, j)] = gfull_t(d, L, i, j);
}

// ---------------------------------------------------------------------------------
// Pointwise and stencil transposes
// ---------------------------------------------------------------------------------
// Drag of the state after a step, scaled: adds s*dCd/dstate (and s*dCd/domega).
__global__ void k_adj_drag(Dev d, Adj a, double s)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j == 1) a.lomega[0] += s * a.DCW[0];
    if (j > d.NJ - 1) return;
    const int c = IDX(1, j);
    a.lP[c] += s * a.DCP[j];
    a.lU[c] += s * a.DCU[j];
    a.lV[c] += s * a.DCV[j];
}

// Correction (Main.f90:97-103): u = u^ + dt S(P)/J.  lW holds the adjoint of the
// corrected interior: adjoint of u^ and of S.
__global__ void k_adj_correct(Dev d, Adj a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    const double f = d.dt / d.DJAC[c];
    a.lSc[c] = f * a.lW[c];
    a.lScV[c] = f * a.lWV[c];
    a.lUh[c] = a.lW[c];
    a.lVh[c] = a.lWV[c];
}

// P_SOURCE transposed (p_source.f90:9-27): S_U(c) = -0.5 sum(+-J xi_x P) over the
// four face neighbours, S_V with xi_y / eta_y.  Scatters into lP (full array).
__global__ void k_adj_psource(Dev d, const double *lSU_, const double *lSV_, double *lP)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    const double au = -0.5 * lSU_[c], av = -0.5 * lSV_[c];
    const double *J = d.DJAC;
    const int e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
    atomicAdd(&lP[e], (J[e] * d.XIX[e]) * au + (J[e] * d.XIY[e]) * av);
    atomicAdd(&lP[w], -((J[w] * d.XIX[w]) * au + (J[w] * d.XIY[w]) * av));
    atomicAdd(&lP[nn], (J[nn] * d.ETX[nn]) * au + (J[nn] * d.ETY[nn]) * av);
    atomicAdd(&lP[s], -((J[s] * d.ETX[s]) * au + (J[s] * d.ETY[s]) * av));
}

// Face fluxes transposed (contra_vel.f90:9-21): UE(c) = 0.5 (J U1)(c) + 0.5 (J U1)(e)
// etc. with U1 = xi_x u + xi_y v, U2 = eta_x u + eta_y v; UW(1,j) = WB(j) blow(j).
__device__ __forceinline__ void flux_scatter(const Dev &d, double *lu, double *lv, int x, double l1, double l2)
{
    // l1: adjoint of (J U1)(x), l2: adjoint of (J U2)(x)
    const double J = d.DJAC[x];
    atomicAdd(&lu[x], J * (d.XIX[x] * l1 + d.ETX[x] * l2));
    atomicAdd(&lv[x], J * (d.XIY[x] * l1 + d.ETY[x] * l2));
}

__global__ void k_adj_flux(Dev d, Adj a, const double *lE, const double *lWf, const double *lN, const double *lS,
                           double *lu, double *lv)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    const double e = 0.5 * lE[c], w = 0.5 * lWf[c], n = 0.5 * lN[c], s = 0.5 * lS[c];
    if (i == 1) {
        a.lblow[j] += d.WB[j] * lWf[c];
        flux_scatter(d, lu, lv, c, e, n + s);
    } else {
        flux_scatter(d, lu, lv, c, e + w, n + s);
        flux_scatter(d, lu, lv, IDX(i - 1, j), w, 0.0);
    }
    flux_scatter(d, lu, lv, IDX(i + 1, j), e, 0.0);
    flux_scatter(d, lu, lv, IDX(i, j + 1), 0.0, n);
    flux_scatter(d, lu, lv, IDX(i, j - 1), 0.0, s);
}

// DIV/dt transposed (iter_p.f90:27-29): flux adjoints from the Poisson adjoint.
__global__ void k_adj_div(Dev d, Adj a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    const double m = d.rdt * a.mu[c];
    a.lFE[c] = m;
    a.lFW[c] = -m;
    a.lFN[c] = m;
    a.lFS[c] = -m;
}

// Cross-derivative term transposed: cross(K,f)(i,j) = 0.25*(K_e(f_ne-f_se) -
// K_w(f_nw-f_sw) + K_n(f_ne-f_nw) - K_s(f_se-f_sw)); scatters L*weights into lf.
__device__ __forceinline__ void cross_scatter(const Dev &d, const double *K, double *lf, int i, int j, double L)
{
    const double ke = K[IDX(i + 1, j)], kw = K[IDX(i - 1, j)], kn = K[IDX(i, j + 1)], ks = K[IDX(i, j - 1)];
    const double q = 0.25 * L;
    atomicAdd(&lf[IDX(i + 1, j + 1)], q * (ke + kn));
    atomicAdd(&lf[IDX(i + 1, j - 1)], -q * (ke + ks));
    atomicAdd(&lf[IDX(i - 1, j + 1)], -q * (kw + kn));
    atomicAdd(&lf[IDX(i - 1, j - 1)], q * (kw + ks));
}

// Second-factor right-hand side transposed (iter_u.f90:86-99 as k_af_su2):
// SU2 = RJDT phi + cross(JYE, phi) + 2 awall wallF (i=1) + 2 afar farF (i=NI-1).
__global__ void k_adj_su2(Dev d, const double *lsu, double *lphi, double *lwall, double *lfar)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    const double L = lsu[c];
    atomicAdd(&lphi[c], d.RJDT[c] * L);
    cross_scatter(d, d.JYE, lphi, i, j, L);
    if (i == 1) lwall[j] += (2.0 * d.cUY.awall[j]) * L;
    if (i == d.NI - 1) lfar[j] += (2.0 * d.cUY.afar[j]) * L;
}

// Explicit phase transposed for one velocity component (Main.f90:61-74 and the
// first-factor right-hand side iter_u.f90:31-46 as af_su1_at):
//   SU1 = (RJDT phi_n - 3Re NL + Re NL_nm1) + DIF(phi_n) + 2Re S + cross(JXE, phi_n)
//         + 2 awall wallF (i=1) + 2 afar farF (i=NI-1)
//   NL  = NL(phi_n; UE, UW, VN, VS)       (bilinear, base point phi_n and fluxes)
//   DIF = D-weighted differences + the cross term of cell (i-1,j-1) (positional)
// lnl: adjoint of the NL computed in this step (in: from the next step, where it is
// NL_nm1; out: the adjoint of this step's NL_nm1 input).  Scatters into lphi (the
// adjoint of phi_n, full array), the flux adjoints, lS (S adjoint), wall/far values.
__global__ void k_adj_explicit(Dev d, Adj a, const double *phin, const double *lsu, double *lnl, double *lphi,
                               double *lS, double *lwall, double *lfar)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    const double L = lsu[c];
    const double rek = d.re;
    // right-hand side assembly
    atomicAdd(&lphi[c], d.RJDT[c] * L);
    const double lnew = lnl[c] - (3.0 * rek) * L;   // adjoint of this step's NL
    lnl[c] = rek * L;                                // adjoint of NL_nm1 (the previous step's NL)
    lS[c] += (2.0 * rek) * L;
    cross_scatter(d, d.JXE, lphi, i, j, L);
    if (i == 1) lwall[j] += (2.0 * d.cUX.awall[j]) * L;
    if (i == d.NI - 1) lfar[j] += (2.0 * d.cUX.afar[j]) * L;
    // DIF (orthogonal part and the cross term)
    {
        const int e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
        atomicAdd(&lphi[e], d.DE[c] * L);
        atomicAdd(&lphi[w], d.DW[c] * L);
        atomicAdd(&lphi[nn], d.DN[c] * L);
        atomicAdd(&lphi[s], d.DS[c] * L);
        atomicAdd(&lphi[c], -(((d.DE[c] + d.DW[c]) + d.DN[c]) + d.DS[c]) * L);
        if (!d.dd_pos) cross_scatter(d, d.JQ12, lphi, i, j, L);
        else if (i > 1 && j > 1) cross_scatter(d, d.JQ12, lphi, i - 1, j - 1, L);
    }
    // NL (nl.f90:21-27): 0.5*UE(p_c+p_e) - 0.5*UW(p_c+p_w) + 0.5*VN(p_c+p_n) - 0.5*VS(p_c+p_s)
    {
        const int e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
        const double h = 0.5 * lnew;
        atomicAdd(&lphi[c], h * (((d.UE[c] - d.UW[c]) + d.VN[c]) - d.VS[c]));
        atomicAdd(&lphi[e], h * d.UE[c]);
        atomicAdd(&lphi[w], -h * d.UW[c]);
        atomicAdd(&lphi[nn], h * d.VN[c]);
        atomicAdd(&lphi[s], -h * d.VS[c]);
        const double pc = phin[c];
        a.lFE[c] += h * (pc + phin[e]);
        a.lFW[c] -= h * (pc + phin[w]);
        a.lFN[c] += h * (pc + phin[nn]);
        a.lFS[c] -= h * (pc + phin[s]);
    }
}

// Far-field values transposed (bcu.f90:27-32 as k_farfield_step): outflow columns
// f(j) = 0.5(q_NI + q_NI-1) - dt*uin*(a (q_NI - q_NI-1) + b dq), inflow constant.
__global__ void k_adj_farfield(Dev d, const double *lfar, double *lq)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > d.NJ - 1) return;
    const int NI = d.NI;
    const double th = d.THETA[IDX(NI, j)];
    if (th >= 0.5 * d.pi && th <= 1.5 * d.pi) return;
    const double L = lfar[j];
    const double a = 0.5 * (d.XIX[IDX(NI, j)] + d.XIX[IDX(NI - 1, j)]);
    const double b = (0.5 * (d.ETX[IDX(NI, j)] + d.ETX[IDX(NI - 1, j)])) * 0.25;
    const double k = d.dt * d.uin;
    atomicAdd(&lq[IDX(NI, j)], (0.5 - k * a) * L);
    atomicAdd(&lq[IDX(NI - 1, j)], (0.5 + k * a) * L);
    atomicAdd(&lq[IDX(NI, j + 1)], -k * b * L);
    atomicAdd(&lq[IDX(NI - 1, j + 1)], -k * b * L);
    atomicAdd(&lq[IDX(NI, j - 1)], k * b * L);
    atomicAdd(&lq[IDX(NI - 1, j - 1)], k * b * L);
}

// Ghost-row refresh of the radial sweep transposed: the ghosts of U* are the
// Dirichlet ghosts of the pre-sweep field (refresh_row_ghosts with BCK_DIRICHLET),
// i.e. k_adj_gd applied to the ghost part only, folded into the pre-sweep
// interior accumulator.
__global__ void k_adj_refresh(Dev d, double *lphi, double *lpre, double *lwall, double *lfar)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    const int NI = d.NI, NJ = d.NJ;
    if (i > NI - 1 || j > NJ - 1) return;
    double s = 0.0;
    if (j == 1) s += lphi[IDX(i, NJ)];
    if (j == NJ - 1) s += lphi[IDX(i, 0)];
    if (i == 1) {
        double g = lphi[IDX(0, j)];
        if (j == 1) g += lphi[IDX(0, NJ)];
        if (j == NJ - 1) g += lphi[IDX(0, 0)];
        s -= g;
        lwall[j] += 2.0 * g;
    }
    if (i == NI - 1) {
        double g = lphi[IDX(NI, j)];
        if (j == 1) g += lphi[IDX(NI, NJ)];
        if (j == NJ - 1) g += lphi[IDX(NI, 0)];
        s -= g;
        lfar[j] += 2.0 * g;
    }
    lpre[IDX(i, j)] += s;
}

// out_int += in_int (interior), then in cleared (full array).
__global__ void k_adj_add_interior(Dev d, double *out, double *in)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    out[IDX(i, j)] += in[IDX(i, j)];
    in[IDX(i, j)] = 0.0;
}

// u^ = u** - dt S/J (Main.f90:80-84): adjoint of u** (interior) and of S.
__global__ void k_adj_grad(Dev d, Adj a, const double *lw, const double *lwv, double *lu, double *lv)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    const double f = d.dt / d.DJAC[c];
    lu[c] = lw[c];
    lv[c] = lwv[c];
    a.lSe[c] -= f * lw[c];
    a.lSeV[c] -= f * lwv[c];
}

// ---------------------------------------------------------------------------------
// Zebra line sweeps transposed.  Forward, a line of one colour is overwritten by
// x = T^{-1} (couplings x other-colour values + rhs); reversed, its adjoint y =
// T^{-T} lam is added to the rhs adjoint, scattered to the other colour with the
// forward coupling coefficients, and the line's own adjoint is cleared.
// ---------------------------------------------------------------------------------
template <int M, int NW>
__global__ void __launch_bounds__(128) k_adj_line_r(Dev d, LineSys s, Coef cf, double *lam, double *lrhs, int colour)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sm[G][TG * M + M * NW + 1];
    __shared__ double xch[G][2 * NW];
    int gl, t, gib;
    group_of<NW>(gl, t, gib);
    const bool active = gl < (d.NJ - 1) / 2;
    const int j = active ? 2 * gl + 1 + colour : 1;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const int n = s.n;
    double v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        v[k] = (active && e < n) ? lam[IDX(e + 1, j)] : 0.0;
    }
    to_chunks<double, M, NW>(v, sm[gib], t);
    const size_t base = size_t(j - 1) * TG * M;
    group_apply<double, M, NW>(v, s.invD + base, s.fa + base, s.fb + base, t, xch[gib]);
    to_interleaved<double, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) {
            const int c = IDX(e + 1, j);
            lrhs[c] += v[k];
            atomicAdd(&lam[IDX(e + 1, jn)], cf.AN[c] * v[k]);
            atomicAdd(&lam[IDX(e + 1, js)], cf.AS[c] * v[k]);
            lam[c] = 0.0;
        }
    }
}

template <int M, int NW>
__global__ void __launch_bounds__(128) k_adj_line_t(Dev d, LineSys s, Coef cf, double *lam, double *lrhs, int colour)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sm[G][TG * M + M * NW + 1];
    __shared__ double xch[G][2 * NW];
    int gl, t, gib;
    group_of<NW>(gl, t, gib);
    const int i0 = 2 * gl + 1 + colour;
    const bool active = i0 <= d.NI - 1;
    const int i = active ? i0 : 1;
    const int n = s.n;
    double v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        v[k] = (active && e < n) ? lam[IDX(i, e + 1)] : 0.0;
    }
    to_chunks<double, M, NW>(v, sm[gib], t);
    const size_t base = size_t(i - 1) * TG * M;
    group_apply<double, M, NW>(v, s.invD + base, s.fa + base, s.fb + base, t, xch[gib]);
    group_cyclic_fix<double, M, NW>(v, s.z + base, s.cv[i - 1], s.sinv[i - 1], n, t, xch[gib]);
    to_interleaved<double, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) {
            const int c = IDX(i, e + 1);
            lrhs[c] += v[k];
            if (cf.AE[c] != 0.0) atomicAdd(&lam[IDX(i + 1, e + 1)], cf.AE[c] * v[k]);
            if (cf.AW[c] != 0.0) atomicAdd(&lam[IDX(i - 1, e + 1)], cf.AW[c] * v[k]);
            lam[c] = 0.0;
        }
    }
}

// ---------------------------------------------------------------------------------
// Poisson adjoint: (A^T + G^T DD^T) mu = g by zebra line Gauss-Seidel on A^T with
// the transposed cross term lagged.
// ---------------------------------------------------------------------------------
// (DD^T mu) at array position (x, y).  The cross term of cell (i,j) is
// dd_p(P, a, b) with (a,b) = (i-1, j-1) when paired by position (zero unless
// i, j > 1) or (i, j); dd_p reads P(a+1,b+1), P(a+1,b-1), P(a-1,b+1), P(a-1,b-1).
__device__ __forceinline__ double qdd(const Dev &d, const double *mu, int x, int y)
{
    const int o = d.dd_pos;
    double q = 0.0;
    auto term = [&](const double *C, int a, int b) {
        const int i = a + o, j = b + o;
        if (a < 1 || b < 1 || i > d.NI - 1 || j > d.NJ - 1) return;
        q += C[IDX(a, b)] * mu[IDX(i, j)];
    };
    term(d.CNE, x - 1, y - 1);
    term(d.CSE, x - 1, y + 1);
    term(d.CNW, x + 1, y - 1);
    term(d.CSW, x + 1, y + 1);
    return q;
}

// G^T DD^T mu at interior cell (i,j) (the BCP ghost map folded as in gfull_t).
__device__ __forceinline__ double xd_at(const Dev &d, const double *mu, int i, int j)
{
    const int NI = d.NI, NJ = d.NJ;
    double s = qdd(d, mu, i, j);
    if (j == NJ - 1) s += qdd(d, mu, i, 0);
    if (j == 1) s += qdd(d, mu, i, NJ);
    if (i == 1) {
        s += qdd(d, mu, 0, j);
        if (j == NJ - 1) s += qdd(d, mu, 0, 0);
        if (j == 1) s += qdd(d, mu, 0, NJ);
    }
    double w = 0.0;
    if (i == NI - 1) w += 3.0;
    if (i == NI - 2) w -= 3.0;
    if (i == NI - 3) w += 1.0;
    if (w != 0.0) {
        double g = qdd(d, mu, NI, j);
        if (j == NJ - 1) g += qdd(d, mu, NI, 0);
        if (j == 1) g += qdd(d, mu, NI, NJ);
        s += w * g;
    }
    return s;
}

// qdd and xd_at in double-float (the same terms in the same order, each FP64
// operand split on load): the mixed path's residual of the transposed equation.
__device__ __forceinline__ dd qdd_df(const Dev &d, const double *mu, int x, int y)
{
    const int o = d.dd_pos;
    dd q(0.0f, 0.0f);
    auto term = [&](const double *C, int a, int b) {
        const int i = a + o, j = b + o;
        if (a < 1 || b < 1 || i > d.NI - 1 || j > d.NJ - 1) return;
        q = q + dd_split(C[IDX(a, b)]) * dd_split(mu[IDX(i, j)]);
    };
    term(d.CNE, x - 1, y - 1);
    term(d.CSE, x - 1, y + 1);
    term(d.CNW, x + 1, y - 1);
    term(d.CSW, x + 1, y + 1);
    return q;
}

__device__ __forceinline__ dd xd_at_df(const Dev &d, const double *mu, int i, int j)
{
    const int NI = d.NI, NJ = d.NJ;
    dd s = qdd_df(d, mu, i, j);
    if (j == NJ - 1) s = s + qdd_df(d, mu, i, 0);
    if (j == 1) s = s + qdd_df(d, mu, i, NJ);
    if (i == 1) {
        s = s + qdd_df(d, mu, 0, j);
        if (j == NJ - 1) s = s + qdd_df(d, mu, 0, 0);
        if (j == 1) s = s + qdd_df(d, mu, 0, NJ);
    }
    float w = 0.0f;
    if (i == NI - 1) w += 3.0f;
    if (i == NI - 2) w -= 3.0f;
    if (i == NI - 3) w += 1.0f;
    if (w != 0.0f) {
        dd g = qdd_df(d, mu, NI, j);
        if (j == NJ - 1) g = g + qdd_df(d, mu, NI, 0);
        if (j == 1) g = g + qdd_df(d, mu, NI, NJ);
        s = s + dd(w, 0.0f) * g;
    }
    return s;
}

__global__ void k_adj_xd(Dev d, Adj a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    if (a.pctl->done) return;
    a.XD[IDX(i, j)] = xd_at(d, a.mu, i, j);
}

template <int M, int NW>
__global__ void __launch_bounds__(128) k_adj_pois(Dev d, Adj a, int colour)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sm[G][TG * M + M * NW + 1];
    __shared__ double xch[G][2 * NW];
    const int stop = a.pctl->done;   // tested after the operand loads
    int gl, t, gib;
    group_of<NW>(gl, t, gib);
    const bool active = gl < (d.NJ - 1) / 2;
    const int j = active ? 2 * gl + 1 + colour : 1;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const LineSys &s = a.sPT;
    const Coef &cf = a.cPT;
    const int n = s.n;
    double v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        v[k] = 0.0;
        if (active && e < n) {
            const int c = IDX(e + 1, j);
            v[k] = ((cf.AN[c] * a.mu[IDX(e + 1, jn)] + cf.AS[c] * a.mu[IDX(e + 1, js)]) + a.g[c]) - a.XD[c];
        }
    }
    if (stop) return;
    to_chunks<double, M, NW>(v, sm[gib], t);
    const size_t base = size_t(j - 1) * TG * M;
    group_apply<double, M, NW>(v, s.invD + base, s.fa + base, s.fb + base, t, xch[gib]);
    to_interleaved<double, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) a.mu[IDX(e + 1, j)] = v[k];
    }
}

// Scaled L1 residual of the transposed equation (cross term of the current mu);
// the last block decides convergence (tolerance tol, cap nmax iterations).
__global__ void __launch_bounds__(256) k_adj_pres(Dev d, Adj a, int per, double tol, int nmax)
{
    __shared__ double sh[64];
    __shared__ bool last;
    if (a.pctl->done) return;
    Dev da = d;
    da.pctl = a.pctl;
    da.partial = a.partial;
    const int ni1 = d.NI - 1, total = ni1 * (d.NJ - 1);
    const Coef &cf = a.cPT;
    double ra = 0.0, pa = 0.0;
#pragma unroll
    for (int q = 0; q < RES_CELLS; q++) {
        int e = (blockIdx.x * RES_CELLS + q) * 256 + threadIdx.x;
        if (e < total) {
            int i = e % ni1 + 1, j = e / ni1 + 1, c = IDX(i, j);
            const double *mu = a.mu;
            double am = cf.AP[c] * mu[c] - cf.AE[c] * mu[IDX(i + 1, j)] - cf.AW[c] * mu[IDX(i - 1, j)] -
                        cf.AN[c] * mu[IDX(i, jwrap(d, j + 1))] - cf.AS[c] * mu[IDX(i, jwrap(d, j - 1))];
            double r = (a.g[c] - xd_at(d, mu, i, j)) - am;
            ra += fabs(r);
            pa += fabs(cf.AP[c] * mu[c]);
        }
    }
    if (!grid_sum2(da, ra, pa, sh, last, d.nblk_res)) return;
    if (threadIdx.x == 0) {
        const int it = a.pctl->niter + per;
        const double resip = pa > 0.0 ? ra / pa : 0.0;
        a.pctl->niter = it;
        a.pctl->resip = resip;
        if (!(resip > tol && it < nmax)) {
            a.pctl->done = 1;
            a.pctl->capped = resip > tol ? 1 : 0;
        }
    }
}

// MIXED: the transposed Poisson equation by defect correction of the FP64 mu around
// FP32 zebra sweeps, as the forward solve.  Each outer iteration forms the residual
// r = g - XD(mu) - A^T mu with the cross term of the current mu in double-float
// (FP32 pairs, ~2^-46 relative per term, as the forward residual), its scaled L1
// norm (the convergence test; FP32 within a warp, FP64 beyond) and r in FP32;
// refine_sweeps FP32 zebra sweeps solve A^T dmu = r from dmu = 0; mu += dmu in FP64.
__global__ void __launch_bounds__(256) k_adj_mres(Dev d, Adj a, double tol, int nmax)
{
    __shared__ double sh[64];
    __shared__ bool last;
    if (a.pctl->done) return;
    Dev da = d;
    da.pctl = a.pctl;
    da.partial = a.partial;
    const int it = a.pctl->niter;
    const int ni1 = d.NI - 1, total = ni1 * (d.NJ - 1);
    const Coef &cf = a.cPT;
    float raf = 0.0f, paf = 0.0f;
#pragma unroll
    for (int q = 0; q < RES_CELLS; q++) {
        int e = (blockIdx.x * RES_CELLS + q) * 256 + threadIdx.x;
        if (e < total) {
            int i = e % ni1 + 1, j = e / ni1 + 1, c = IDX(i, j);
            const double *mu = a.mu;
            const dd app = dd_split(cf.AP[c]) * dd_split(mu[c]);
            const dd am = (((app - dd_split(cf.AE[c]) * dd_split(mu[IDX(i + 1, j)])) -
                            dd_split(cf.AW[c]) * dd_split(mu[IDX(i - 1, j)])) -
                           dd_split(cf.AN[c]) * dd_split(mu[IDX(i, jwrap(d, j + 1))])) -
                          dd_split(cf.AS[c]) * dd_split(mu[IDX(i, jwrap(d, j - 1))]);
            const dd r = (dd_split(a.g[c]) - xd_at_df(d, mu, i, j)) - am;
            raf += fabsf(r.hi);
            paf += fabsf(app.hi);
            d.RF[c] = r.hi;
            d.DF[c] = 0.0f;
        }
    }
    double ra, pa;
    if (!grid_sum2f(da, raf, paf, ra, pa, sh, last, d.nblk_res)) return;
    if (threadIdx.x == 0) {
        const double resip = pa > 0.0 ? ra / pa : 0.0;
        a.pctl->resip = resip;
        if (it > 0 && !(resip > tol && it < nmax)) {
            a.pctl->done = 1;
            a.pctl->capped = resip > tol ? 1 : 0;
        } else {
            a.pctl->niter = it + d.refine_sweeps;
        }
    }
}

template <int M, int NW>
__global__ void __launch_bounds__(128) k_adj_pois32(Dev d, Adj a, int colour)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ float sm[G][TG * M + M * NW + 1];
    __shared__ float xch[G][2 * NW];
    const int stop = a.pctl->done;   // tested after the operand loads
    int gl, t, gib;
    group_of<NW>(gl, t, gib);
    const bool active = gl < (d.NJ - 1) / 2;
    const int j = active ? 2 * gl + 1 + colour : 1;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const LineSys &s = a.sPT;
    const Coef &cf = a.cPT;
    const int n = s.n;
    float v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        v[k] = 0.0f;
        if (active && e < n) {
            const int c = IDX(e + 1, j);
            v[k] = (cf.ANf[c] * d.DF[IDX(e + 1, jn)] + cf.ASf[c] * d.DF[IDX(e + 1, js)]) + d.RF[c];
        }
    }
    if (stop) return;
    to_chunks<float, M, NW>(v, sm[gib], t);
    const size_t base = size_t(j - 1) * TG * M;
    group_apply<float, M, NW>(v, s.invDf + base, s.faf + base, s.fbf + base, t, xch[gib]);
    to_interleaved<float, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) d.DF[IDX(e + 1, j)] = v[k];
    }
}

__global__ void k_adj_apply(Dev d, Adj a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    if (a.pctl->done) return;
    const int c = IDX(i, j);
    a.mu[c] = a.mu[c] + (double)d.DF[c];
}

__global__ void k_adj_coef_f32(Dev d, Coef cf)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const int c = IDX(i, j);
    cf.ANf[c] = (float)cf.AN[c];
    cf.ASf[c] = (float)cf.AS[c];
}

__global__ void k_adj_pctl_reset(Adj a)
{
    a.pctl->niter = 0;
    a.pctl->done = 0;
    a.pctl->capped = 0;
    a.pctl->fault = 0;
    a.pctl->resip = 0.0;
}

// Controls from the wall-value adjoints: UFW = -omega sin th + b cos th,
// VFW = omega cos th + b sin th (th = THETA(0,j)); out[0] = dJ/domega,
// out[j] = dJ/db_j (j = 1..NJ-1).
__global__ void k_adj_controls(Dev d, Adj a, double *out)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > d.NJ - 1) return;
    if (j == 0) {
        double s = a.lomega[0];
        for (int k = 1; k <= d.NJ - 1; k++) {
            const double th = d.THETA[IDX(0, k)];
            s += -sin(th) * a.lUFW[k] + cos(th) * a.lVFW[k];
        }
        out[0] = s;
        return;
    }
    const double th = d.THETA[IDX(0, j)];
    out[j] = (cos(th) * a.lUFW[j] + sin(th) * a.lVFW[j]) + a.lblow[j];
}

}  // namespace
}  // namespace fvm

// ---------------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------------
struct fvm_adj {
    fvm::Adj a{};
    char *slab = nullptr;
    double *ctrl = nullptr;              // device: control gradient (1 + NJ-1)
    double *ckpt = nullptr;              // checkpoints: nckpt x 7 full arrays
    double *base = nullptr;              // U, V before every step of a segment: seg x 2 full arrays
    double *fin = nullptr;               // state at the end of the window: 7 full arrays
    int nckpt = 0, nseg_steps = 0;
    cudaGraphExec_t pgraph = nullptr;    // adjoint Poisson loop body
    int pgraph_iters = 0;
    fvm::PCtl *h_pctl = nullptr;
    long long adj_sweeps = 0;
};

namespace fvm {
namespace {

#define ARC(x)                \
    do {                      \
        int rc_ = (x);        \
        if (rc_) return rc_;  \
    } while (0)

inline dim3 igrid(const fvm_ctx *c) { return dim3((c->NI - 1 + 127) / 128, c->NJ - 1); }

void carve_coef_t(char *&p, Coef &cf, size_t n)
{
    auto take = [&](size_t cnt) {
        p = (char *)(((uintptr_t)p + 255) & ~uintptr_t(255));
        double *r = (double *)p;
        p += cnt * sizeof(double);
        return r;
    };
    cf.AP = take(n);
    cf.AE = take(n);
    cf.AW = take(n);
    cf.AN = take(n);
    cf.AS = take(n);
    cf.ANf = reinterpret_cast<float *>(take((n + 1) / 2));
    cf.ASf = reinterpret_cast<float *>(take((n + 1) / 2));
}

void carve_sys_t(char *&p, LineSys &s, const LineSys &like)
{
    s = like;
    const size_t cnt = size_t(like.lines) * WARP * like.NW * like.M;
    auto take = [&](size_t k) {
        p = (char *)(((uintptr_t)p + 255) & ~uintptr_t(255));
        double *r = (double *)p;
        p += k * sizeof(double);
        return r;
    };
    s.invD = take(cnt);
    s.fa = take(cnt);
    s.fb = take(cnt);
    s.invDf = reinterpret_cast<float *>(take((cnt + 1) / 2));   // FP32 factors (mixed Poisson adjoint)
    s.faf = reinterpret_cast<float *>(take((cnt + 1) / 2));
    s.fbf = reinterpret_cast<float *>(take((cnt + 1) / 2));
    s.zf = nullptr;
    s.cvf = nullptr;
    s.sinvf = nullptr;
    if (like.cyclic) {
        s.z = take(cnt);
        s.cv = take(like.lines);
        s.sinv = take(like.lines);
    } else {
        s.z = s.cv = s.sinv = nullptr;
    }
}

// Factors of a transposed set in the layout of `like` (k_factor needs FP32 copies:
// they go to scratch that is not used afterwards).
__global__ void k_adj_factor(Dev d, Coef cf, LineSys s, int circ)
{
    int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= s.lines) return;
    const int n = s.n, M = s.M, TG = WARP * s.NW;
    const size_t base = size_t(line) * TG * M;
    auto at = [&](int e) { return IDX(circ ? line + 1 : e + 1, circ ? e + 1 : line + 1); };
    auto slot = [&](int e) { return base + size_t(e % M) * TG + (e / M); };
    double gamma = 0.0, a1 = 0.0, cn = 0.0;
    if (circ) {
        gamma = -cf.AP[at(0)];
        a1 = -cf.AS[at(0)];
        cn = -cf.AN[at(n - 1)];
    }
    double Bprev = 0.0;
    for (int e = 0; e < n; e++) {
        int c = at(e);
        double a = circ ? -cf.AS[c] : -cf.AW[c];
        double b = cf.AP[c];
        double cc = circ ? -cf.AN[c] : -cf.AE[c];
        if (circ && e == 0) { a = 0.0; b = b - gamma; }
        if (circ && e == n - 1) { b = b - a1 * cn / gamma; cc = 0.0; }
        if (!circ && e == 0) a = 0.0;
        if (!circ && e == n - 1) cc = 0.0;
        double D = b - a * Bprev;
        double B = cc / D;
        size_t k = slot(e);
        s.invD[k] = 1.0 / D;
        s.fa[k] = -a / D;
        s.fb[k] = -B;
        Bprev = B;
    }
    for (int e = n; e < TG * M; e++) {
        size_t k = slot(e);
        s.invD[k] = 0.0;
        s.fa[k] = 0.0;
        s.fb[k] = 0.0;
    }
    for (int e = 0; e < TG * M; e++) {
        size_t k = slot(e);
        s.invDf[k] = (float)s.invD[k];
        s.faf[k] = (float)s.fa[k];
        s.fbf[k] = (float)s.fb[k];
    }
    if (circ) {
        double y = 0.0;
        for (int e = 0; e < n; e++) {
            double u = (e == 0) ? gamma : (e == n - 1 ? cn : 0.0);
            size_t k = slot(e);
            y = s.fa[k] * y + s.invD[k] * u;
            s.z[k] = y;
        }
        double x = 0.0;
        for (int e = n - 1; e >= 0; e--) {
            size_t k = slot(e);
            x = s.z[k] + s.fb[k] * x;
            s.z[k] = x;
        }
        for (int e = n; e < TG * M; e++) s.z[slot(e)] = 0.0;
        double cv = a1 / gamma;
        double z1 = s.z[slot(0)], zn = s.z[slot(n - 1)];
        s.cv[line] = cv;
        s.sinv[line] = 1.0 / (1.0 + z1 + cv * zn);
    }
}

int adj_setup(fvm_ctx *c)
{
    if (c->adj) return FVM_OK;
    fvm_adj *A = new (std::nothrow) fvm_adj();
    if (!A) return FVM_ERR_NOMEM;
    Dev &d = c->d;
    const size_t n = c->n;
    // device slab: 30 full arrays, 8 per-j arrays, 3 transposed sets and factors
    const size_t nj1 = c->NJ + 1;
    auto sys_bytes = [](const LineSys &s) {
        size_t cnt = size_t(s.lines) * WARP * s.NW * s.M;
        // invD, fa, fb, z (FP64), their FP32 copies, cv, sinv, alignment
        return (6 * cnt + 2 * s.lines) * sizeof(double) + 16 * 256;
    };
    // per transposed set: AP, AE, AW, AN, AS (FP64) and ANf, ASf (FP32)
    size_t bytes = (30 * n + 10 * nj1 + 16) * sizeof(double) + 3 * (6 * n * sizeof(double) + 8 * 256) +
                   sys_bytes(d.sP) + sys_bytes(d.sUX) + sys_bytes(d.sUY) + 64 * 256 + sizeof(PCtl) +
                   2 * size_t(c->nblk_res) * sizeof(double);
    cudaError_t e = cudaMalloc(&A->slab, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(A->slab, 0, bytes, c->stream);
    if (e == cudaSuccess) e = cudaMallocHost(&A->h_pctl, sizeof(PCtl));
    if (e != cudaSuccess) {
        if (A->slab) cudaFree(A->slab);
        delete A;
        c->err = std::string("adjoint allocation: ") + cudaGetErrorString(e);
        return FVM_ERR_NOMEM;
    }
    char *p = A->slab;
    auto take = [&](size_t cnt) {
        p = (char *)(((uintptr_t)p + 255) & ~uintptr_t(255));
        double *r = (double *)p;
        p += cnt * sizeof(double);
        return r;
    };
    Adj &a = A->a;
    double **full[] = {&a.lU, &a.lV, &a.lP, &a.lNLX, &a.lNLY, &a.lUn, &a.lVn, &a.lW, &a.lWV, &a.lSc, &a.lScV,
                       &a.lSe, &a.lSeV, &a.lPf, &a.g, &a.mu, &a.XD, &a.lUh, &a.lVh, &a.lSU, &a.lSUV, &a.lFE,
                       &a.lFW, &a.lFN, &a.lFS};
    for (auto q : full) *q = take(n);
    double **perj[] = {&a.lUFW, &a.lVFW, &a.lFFU, &a.lFFV, &a.lblow, &a.DCU, &a.DCV, &a.DCP};
    for (auto q : perj) *q = take(nj1);
    a.lomega = take(2);
    a.DCW = take(2);
    A->ctrl = take(nj1);
    carve_coef_t(p, a.cPT, n);
    carve_coef_t(p, a.cXT, n);
    carve_coef_t(p, a.cYT, n);
    carve_sys_t(p, a.sPT, d.sP);
    carve_sys_t(p, a.sXT, d.sUX);
    carve_sys_t(p, a.sYT, d.sUY);
    p = (char *)(((uintptr_t)p + 255) & ~uintptr_t(255));
    a.pctl = (PCtl *)p;
    p += sizeof(PCtl);
    a.partial = take(2 * size_t(c->nblk_res));
    if ((size_t)(p - A->slab) > bytes) {
        cudaFree(A->slab);
        cudaFreeHost(A->h_pctl);
        delete A;
        c->err = "adjoint slab overflow";
        return FVM_ERR_ARG;
    }
    // transposed coefficient sets and their factors, drag sensitivities
    k_adj_coef_t<<<igrid(c), 128, 0, c->stream>>>(d, d.cP, a.cPT);
    k_adj_coef_f32<<<igrid(c), 128, 0, c->stream>>>(d, a.cPT);
    k_adj_coef_t<<<igrid(c), 128, 0, c->stream>>>(d, d.cUX, a.cXT);
    k_adj_coef_t<<<igrid(c), 128, 0, c->stream>>>(d, d.cUY, a.cYT);
    k_adj_factor<<<(a.sPT.lines + 63) / 64, 64, 0, c->stream>>>(d, a.cPT, a.sPT, 0);
    k_adj_factor<<<(a.sXT.lines + 63) / 64, 64, 0, c->stream>>>(d, a.cXT, a.sXT, 0);
    k_adj_factor<<<(a.sYT.lines + 63) / 64, 64, 0, c->stream>>>(d, a.cYT, a.sYT, 1);
    k_adj_dragcoef<<<(c->NJ + 127) / 128, 128, 0, c->stream>>>(d, a);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cudaFree(A->slab);
        cudaFreeHost(A->h_pctl);
        delete A;
        c->err = std::string("adjoint setup: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    c->adj = A;
    return FVM_OK;
}

// Adjoint Poisson loop body: `groups` x (res_every x [cross term, colour 0,
// colour 1], residual), captured once, replayed until converged.
int adj_poisson_graph(fvm_ctx *c)
{
    fvm_adj *A = c->adj;
    if (A->pgraph) return FVM_OK;
    const Dev &d = c->d;
    const Adj &a = A->a;
    const bool mixed = c->p.precision == FVM_MIXED;
    const int per = mixed ? c->d.refine_sweeps : 4, groups = mixed ? std::max(1, 32 / per) : 8;
    cudaGraph_t g = nullptr;
    FVM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int blocks = line_blocks((c->NJ - 1) / 2, a.sPT.NW);
    bool ok = true;
    // the transposed FP32 correction: in the forward solve's resident kernel when the
    // context uses it (its transposed factors share the forward tile), else per colour
    const ResSys sys{a.sPT.invDf, a.sPT.faf, a.sPT.fbf, a.cPT.ANf, a.cPT.ASf, d.RF, d.DF, a.mu, a.pctl, 0};
    for (int q = 0; q < groups && ok && mixed && c->res_lines; q++) {
        k_adj_mres<<<c->nblk_res, 256, 0, c->stream>>>(d, a, c->p.resimax, c->d.nswpp);
        int rc = resident_sweeps_on(c, sys, per, 1, 1);
        if (rc) {
            cudaGraph_t gg = nullptr;
            cudaStreamEndCapture(c->stream, &gg);
            if (gg) cudaGraphDestroy(gg);
            return rc;
        }
    }
    for (int q = 0; q < groups && ok && mixed && !c->res_lines; q++) {
        k_adj_mres<<<c->nblk_res, 256, 0, c->stream>>>(d, a, c->p.resimax, c->d.nswpp);
        for (int it = 0; it < per && ok; it++)
            for (int colour = 0; colour < 2; colour++)
                ok = ok && dispatch_line(a.sPT, [&](auto m, auto nw) {
                         k_adj_pois32<decltype(m)::value, decltype(nw)::value>
                             <<<blocks, 128, 0, c->stream>>>(d, a, colour);
                     });
        k_adj_apply<<<igrid(c), 128, 0, c->stream>>>(d, a);
    }
    for (int q = 0; q < groups && ok && !mixed; q++) {
        for (int it = 0; it < per && ok; it++) {
            k_adj_xd<<<igrid(c), 128, 0, c->stream>>>(d, a);
            for (int colour = 0; colour < 2; colour++)
                ok = ok && dispatch_line(a.sPT, [&](auto m, auto nw) {
                         k_adj_pois<decltype(m)::value, decltype(nw)::value>
                             <<<blocks, 128, 0, c->stream>>>(d, a, colour);
                     });
        }
        k_adj_pres<<<c->nblk_res, 256, 0, c->stream>>>(d, a, per, c->p.resimax, c->d.nswpp);
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (!ok || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        c->err = ok ? std::string("adjoint Poisson capture: ") + cudaGetErrorString(e) : "unsupported line length";
        return ok ? FVM_ERR_CUDA : FVM_ERR_ARG;
    }
    e = cudaGraphInstantiate(&A->pgraph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->err = std::string("adjoint Poisson instantiate: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    A->pgraph_iters = per * groups;
    return FVM_OK;
}

int adj_poisson(fvm_ctx *c)
{
    fvm_adj *A = c->adj;
    ARC(adj_poisson_graph(c));
    k_adj_pctl_reset<<<1, 1, 0, c->stream>>>(A->a);
    const long max_launches = (long)c->d.nswpp / A->pgraph_iters + 2;
    for (long l = 0;; l++) {
        if (l >= max_launches) {
            c->err = "adjoint Poisson iteration did not report completion within the sweep cap";
            return FVM_ERR_TIMEOUT;
        }
        FVM_CUDA(c, cudaGraphLaunch(A->pgraph, c->stream));
        FVM_CUDA(c, cudaMemcpyAsync(A->h_pctl, A->a.pctl, sizeof(PCtl), cudaMemcpyDeviceToHost, c->stream));
        FVM_CUDA(c, cudaStreamSynchronize(c->stream));
        if (A->h_pctl->done) break;
    }
    A->adj_sweeps += A->h_pctl->niter;
    if (A->h_pctl->fault) {   // a bounded wait of the resident sweeps ran out
        ARC(resident_reset(c));
        FVM_CUDA(c, cudaMemsetAsync(&A->a.pctl->fault, 0, sizeof(int), c->stream));
        FVM_CUDA(c, cudaStreamSynchronize(c->stream));
        c->err = "adjoint Poisson: a bounded wait of the resident sweeps ran out";
        return FVM_ERR_TIMEOUT;
    }
    if (!std::isfinite(A->h_pctl->resip)) {
        c->err = "non-finite adjoint Poisson residual";
        return FVM_ERR_NAN;
    }
    return FVM_OK;
}

int line_r(fvm_ctx *c, const LineSys &sT, const Coef &cf, double *lam, double *lrhs, int colour)
{
    const int blocks = line_blocks((c->NJ - 1) / 2, sT.NW);
    bool ok = dispatch_line(sT, [&](auto m, auto nw) {
        k_adj_line_r<decltype(m)::value, decltype(nw)::value>
            <<<blocks, 128, 0, c->stream>>>(c->d, sT, cf, lam, lrhs, colour);
    });
    if (!ok) {
        c->err = "unsupported line length";
        return FVM_ERR_ARG;
    }
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int line_t(fvm_ctx *c, const LineSys &sT, const Coef &cf, double *lam, double *lrhs, int colour)
{
    const int blocks = line_blocks((c->NI - 1 + 1 - colour) / 2, sT.NW);
    bool ok = dispatch_line(sT, [&](auto m, auto nw) {
        k_adj_line_t<decltype(m)::value, decltype(nw)::value>
            <<<blocks, 128, 0, c->stream>>>(c->d, sT, cf, lam, lrhs, colour);
    });
    if (!ok) {
        c->err = "unsupported line length";
        return FVM_ERR_ARG;
    }
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

// The predictor of one velocity component transposed: lam holds the adjoint of
// u** (interior, ghosts zero) on entry; on exit lsu holds the adjoint of the
// first-factor right-hand side and lpre has gained the adjoint of the pre-sweep
// field (u^n as the sweeps' initial iterate and the source of their ghost rows).
int adj_predictor(fvm_ctx *c, double *lam, double *lsu, double *lpre, double *lwall, double *lfar)
{
    fvm_adj *A = c->adj;
    const Adj &a = A->a;
    const Dev &d = c->d;
    const size_t bytes = sizeof(double) * c->n;
    FVM_CUDA(c, cudaMemsetAsync(lsu, 0, bytes, c->stream));
    ARC(line_t(c, a.sYT, d.cUY, lam, lsu, 1));
    ARC(line_t(c, a.sYT, d.cUY, lam, lsu, 0));
    k_adj_su2<<<igrid(c), 128, 0, c->stream>>>(d, lsu, lam, lwall, lfar);
    k_adj_refresh<<<igrid(c), 128, 0, c->stream>>>(d, lam, lpre, lwall, lfar);
    k_adj_clear_ghosts<<<(std::max(c->NI, c->NJ) + 1 + 127) / 128, 128, 0, c->stream>>>(d, lam);
    FVM_CUDA(c, cudaMemsetAsync(lsu, 0, bytes, c->stream));
    ARC(line_r(c, a.sXT, d.cUX, lam, lsu, 1));
    ARC(line_r(c, a.sXT, d.cUX, lam, lsu, 0));
    k_adj_add_interior<<<igrid(c), 128, 0, c->stream>>>(d, lpre, lam);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

// One step reversed.  On entry a.lU, lV, lP, lNLX, lNLY hold the adjoint of the
// state after the step; ubase/vbase the U, V of the state before it (full arrays).
// drag_scale: weight of this step's drag coefficient in the objective.
int adj_step(fvm_ctx *c, const double *ubase, const double *vbase, double drag_scale)
{
    fvm_adj *A = c->adj;
    const Adj &a = A->a;
    Dev &d = c->d;
    cudaStream_t st = c->stream;
    const size_t bytes = sizeof(double) * c->n, jb = sizeof(double) * (c->NJ + 1);
    const dim3 G = igrid(c);
    const int rows = (c->NJ + 127) / 128;
    FVM_CUDA(c, cudaMemsetAsync(a.lFFU, 0, jb, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lFFV, 0, jb, st));
    // CALCCOEF of the state after the step
    if (drag_scale != 0.0) k_adj_drag<<<rows, 128, 0, st>>>(d, a, drag_scale);
    // correction and BCU/BCV (Main.f90:97-107)
    k_adj_gd<<<G, 128, 0, st>>>(d, a.lU, a.lW, a.lUFW, a.lFFU, 1);
    k_adj_gd<<<G, 128, 0, st>>>(d, a.lV, a.lWV, a.lVFW, a.lFFV, 1);
    FVM_CUDA(c, cudaMemsetAsync(a.lUh, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lVh, 0, bytes, st));
    k_adj_correct<<<G, 128, 0, st>>>(d, a);
    FVM_CUDA(c, cudaMemcpyAsync(a.lPf, a.lP, bytes, cudaMemcpyDeviceToDevice, st));
    k_adj_psource<<<G, 128, 0, st>>>(d, a.lSc, a.lScV, a.lPf);
    k_adj_gfull<<<G, 128, 0, st>>>(d, a.lPf, a.g);
    FVM_LAUNCH_CHECK(c);
    // ITER_P (converged) and its source DIV/dt
    ARC(adj_poisson(c));
    k_adj_div<<<G, 128, 0, st>>>(d, a);
    k_adj_flux<<<G, 128, 0, st>>>(d, a, a.lFE, a.lFW, a.lFN, a.lFS, a.lUh, a.lVh);
    // u^ = u** - dt S/J with BCU/BCV (Main.f90:80-87)
    k_adj_gd<<<G, 128, 0, st>>>(d, a.lUh, a.lW, a.lUFW, a.lFFU, 1);
    k_adj_gd<<<G, 128, 0, st>>>(d, a.lVh, a.lWV, a.lVFW, a.lFFV, 1);
    FVM_CUDA(c, cudaMemsetAsync(a.lSe, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lSeV, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lU, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lV, 0, bytes, st));
    k_adj_grad<<<G, 128, 0, st>>>(d, a, a.lW, a.lWV, a.lU, a.lV);
    FVM_LAUNCH_CHECK(c);
    // predictors (ITER_U, ITER_V)
    FVM_CUDA(c, cudaMemsetAsync(a.lUn, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lVn, 0, bytes, st));
    ARC(adj_predictor(c, a.lU, a.lSU, a.lUn, a.lUFW, a.lFFU));
    ARC(adj_predictor(c, a.lV, a.lSUV, a.lVn, a.lVFW, a.lFFV));
    // explicit phase at the base point: fluxes of u^n
    FVM_CUDA(c, cudaMemcpyAsync(d.U, ubase, bytes, cudaMemcpyDeviceToDevice, st));
    FVM_CUDA(c, cudaMemcpyAsync(d.V, vbase, bytes, cudaMemcpyDeviceToDevice, st));
    run_contra_vel(c);
    FVM_CUDA(c, cudaMemsetAsync(a.lFE, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lFW, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lFN, 0, bytes, st));
    FVM_CUDA(c, cudaMemsetAsync(a.lFS, 0, bytes, st));
    k_adj_explicit<<<G, 128, 0, st>>>(d, a, ubase, a.lSU, a.lNLX, a.lUn, a.lSe, a.lUFW, a.lFFU);
    k_adj_explicit<<<G, 128, 0, st>>>(d, a, vbase, a.lSUV, a.lNLY, a.lVn, a.lSeV, a.lVFW, a.lFFV);
    FVM_CUDA(c, cudaMemsetAsync(a.lP, 0, bytes, st));
    k_adj_psource<<<G, 128, 0, st>>>(d, a.lSe, a.lSeV, a.lP);
    k_adj_flux<<<G, 128, 0, st>>>(d, a, a.lFE, a.lFW, a.lFN, a.lFS, a.lUn, a.lVn);
    k_adj_farfield<<<rows, 128, 0, st>>>(d, a.lFFU, a.lUn);
    k_adj_farfield<<<rows, 128, 0, st>>>(d, a.lFFV, a.lVn);
    FVM_LAUNCH_CHECK(c);
    FVM_CUDA(c, cudaMemcpyAsync(a.lU, a.lUn, bytes, cudaMemcpyDeviceToDevice, st));
    FVM_CUDA(c, cudaMemcpyAsync(a.lV, a.lVn, bytes, cudaMemcpyDeviceToDevice, st));
    return FVM_OK;
}

int adj_zero(fvm_ctx *c)
{
    const Adj &a = c->adj->a;
    const size_t bytes = sizeof(double) * c->n, jb = sizeof(double) * (c->NJ + 1);
    double *full[] = {a.lU, a.lV, a.lP, a.lNLX, a.lNLY, a.mu};
    for (double *p : full) FVM_CUDA(c, cudaMemsetAsync(p, 0, bytes, c->stream));
    double *perj[] = {a.lUFW, a.lVFW, a.lblow};
    for (double *p : perj) FVM_CUDA(c, cudaMemsetAsync(p, 0, jb, c->stream));
    FVM_CUDA(c, cudaMemsetAsync(a.lomega, 0, 2 * sizeof(double), c->stream));
    return FVM_OK;
}

int adj_controls(fvm_ctx *c, double *dJ_domega, double *dJ_dblow)
{
    fvm_adj *A = c->adj;
    k_adj_controls<<<(c->NJ + 127) / 128, 128, 0, c->stream>>>(c->d, A->a, A->ctrl);
    FVM_LAUNCH_CHECK(c);
    std::vector<double> h(c->NJ + 1);
    FVM_CUDA(c, cudaMemcpyAsync(h.data(), A->ctrl, sizeof(double) * c->NJ, cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (dJ_domega) *dJ_domega = h[0];
    if (dJ_dblow)
        for (int j = 1; j <= c->NJ - 1; j++) dJ_dblow[j - 1] = h[j];
    return FVM_OK;
}

// State arrays a step reads from its predecessor.
int state_copy(fvm_ctx *c, double *buf, bool save)
{
    Dev &d = c->d;
    double *arr[] = {d.U, d.V, d.P, d.T, d.NLX, d.NLY, d.ADV};
    const size_t n = c->n, bytes = sizeof(double) * n;
    for (int k = 0; k < 7; k++) {
        if (save) FVM_CUDA(c, cudaMemcpyAsync(buf + k * n, arr[k], bytes, cudaMemcpyDeviceToDevice, c->stream));
        else FVM_CUDA(c, cudaMemcpyAsync(arr[k], buf + k * n, bytes, cudaMemcpyDeviceToDevice, c->stream));
    }
    return FVM_OK;
}

}  // namespace

int run_adjoint(fvm_ctx *c, int window, int ckpt, double *J, double *dJ_domega, double *dJ_dblow)
{
    ARC(adj_setup(c));
    fvm_adj *A = c->adj;
    const size_t n = c->n;
    const int nck = (window + ckpt - 1) / ckpt;
    if (A->nckpt < nck || A->nseg_steps < ckpt) {
        if (A->ckpt) cudaFree(A->ckpt);
        if (A->base) cudaFree(A->base);
        if (A->fin) cudaFree(A->fin);
        A->ckpt = A->base = A->fin = nullptr;
        FVM_CUDA(c, cudaMalloc(&A->ckpt, sizeof(double) * 7 * n * nck));
        FVM_CUDA(c, cudaMalloc(&A->base, sizeof(double) * 2 * n * ckpt));
        FVM_CUDA(c, cudaMalloc(&A->fin, sizeof(double) * 7 * n));
        A->nckpt = nck;
        A->nseg_steps = ckpt;
    }
    std::vector<double> ck_time(nck);
    std::vector<int> ck_iter(nck);
    // forward pass with checkpoints
    double jsum = 0.0;
    int status = FVM_OK;
    for (int s = 0; s < window; s++) {
        if (s % ckpt == 0) {
            ARC(state_copy(c, A->ckpt + size_t(s / ckpt) * 7 * n, true));
            ck_time[s / ckpt] = c->rtime;
            ck_iter[s / ckpt] = c->niter_time;
        }
        fvm_coeffs co;
        int rc = run_step(c, 1, &co);
        if (rc == FVM_ERR_NOCONV) status = rc;
        else if (rc) return rc;
        jsum += co.cd;
    }
    if (J) *J = jsum / window;
    ARC(state_copy(c, A->fin, true));
    const double t_end = c->rtime;
    const int it_end = c->niter_time;
    const fvm_coeffs last_end = c->last;
    // the recomputation passes repeat steps already taken: no post-processing
    struct Suspend {
        fvm_ctx *c;
        explicit Suspend(fvm_ctx *cc) : c(cc) { c->post_suspend++; }
        ~Suspend() { c->post_suspend--; }
    } suspend(c);
    // reverse pass, one segment at a time
    ARC(adj_zero(c));
    for (int seg = nck - 1; seg >= 0; seg--) {
        ARC(state_copy(c, A->ckpt + size_t(seg) * 7 * n, false));
        c->rtime = ck_time[seg];
        c->niter_time = ck_iter[seg];
        const int s0 = seg * ckpt, s1 = std::min(window, s0 + ckpt);
        for (int s = s0; s < s1; s++) {
            double *b = A->base + size_t(s - s0) * 2 * n;
            FVM_CUDA(c, cudaMemcpyAsync(b, c->d.U, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
            FVM_CUDA(c, cudaMemcpyAsync(b + n, c->d.V, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
            fvm_coeffs co;
            int rc = run_step(c, 1, &co);
            if (rc && rc != FVM_ERR_NOCONV) return rc;
        }
        for (int s = s1 - 1; s >= s0; s--) {
            double *b = A->base + size_t(s - s0) * 2 * n;
            ARC(adj_step(c, b, b + n, 1.0 / window));
        }
    }
    ARC(adj_controls(c, dJ_domega, dJ_dblow));
    ARC(state_copy(c, A->fin, false));
    c->rtime = t_end;
    c->niter_time = it_end;
    c->last = last_end;
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    return status;
}

// Transpose of one step at the context's current state (no drag term): lam (5
// host arrays U, V, P, NLX, NLY) holds the adjoint of the state after the step on
// entry and of the state before it on exit; dctrl gets the control adjoint.
int run_adjoint_vjp(fvm_ctx *c, double *const *lam, double *dctrl)
{
    ARC(adj_setup(c));
    fvm_adj *A = c->adj;
    const Adj &a = A->a;
    const size_t n = c->n, bytes = sizeof(double) * n;
    if (!A->fin) FVM_CUDA(c, cudaMalloc(&A->fin, sizeof(double) * 7 * n));
    double *ub = nullptr;
    FVM_CUDA(c, cudaMalloc(&ub, 2 * bytes));
    int rc = FVM_OK;
    do {
        if ((rc = state_copy(c, A->fin, true))) break;
        if ((rc = adj_zero(c))) break;
        if (cudaMemcpyAsync(ub, c->d.U, bytes, cudaMemcpyDeviceToDevice, c->stream) ||
            cudaMemcpyAsync(ub + n, c->d.V, bytes, cudaMemcpyDeviceToDevice, c->stream)) { rc = FVM_ERR_CUDA; break; }
        double *dst[] = {a.lU, a.lV, a.lP, a.lNLX, a.lNLY};
        for (int k = 0; k < 5 && !rc; k++)
            if (cudaMemcpyAsync(dst[k], lam[k], bytes, cudaMemcpyHostToDevice, c->stream)) rc = FVM_ERR_CUDA;
        if (rc) break;
        // the step's own forward values (fluxes of u^n) are recomputed inside
        if ((rc = adj_step(c, ub, ub + n, 0.0))) break;
        for (int k = 0; k < 5 && !rc; k++)
            if (cudaMemcpyAsync(lam[k], dst[k], bytes, cudaMemcpyDeviceToHost, c->stream)) rc = FVM_ERR_CUDA;
        if (rc) break;
        rc = adj_controls(c, dctrl, dctrl ? dctrl + 1 : nullptr);
        if (rc) break;
        rc = state_copy(c, A->fin, false);
    } while (false);
    cudaStreamSynchronize(c->stream);
    cudaFree(ub);
    return rc;
}

void adj_destroy(fvm_ctx *c)
{
    fvm_adj *A = c->adj;
    if (!A) return;
    if (A->pgraph) cudaGraphExecDestroy(A->pgraph);
    if (A->slab) cudaFree(A->slab);
    if (A->ckpt) cudaFree(A->ckpt);
    if (A->base) cudaFree(A->base);
    if (A->fin) cudaFree(A->fin);
    if (A->h_pctl) cudaFreeHost(A->h_pctl);
    delete A;
    c->adj = nullptr;
}

}  // namespace fvm
