// fvm_step.cu -- the per-step kernels of the GB300 cylinder time step (FP64 path):
// explicit right-hand sides, approximate-factorisation predictor line sweeps,
// projection, the zebra line Gauss-Seidel Poisson iteration, correction, passive
// temperature and the wall-force diagnostics.
//
// Ordering ("GPU order"): identical to the reference's call sequence
// (Main.f90:48-114) and ghost-cell semantics except that every line sweep is
// zebra-ordered (odd lines, then even lines), neighbours across the branch cut
// are read through periodic index wrap inside sweeps and Poisson residuals, and
// the predictor's circumferential lines are solved as cyclic systems.
#include <cmath>
#include <cstring>

#include "fvm_internal.cuh"

namespace fvm {

// ---------------------------------------------------------------------------------
// Cell operators (shared by the per-routine and the fused kernels)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double nl_at(const Dev &d, const double *in, int i, int j)
{   // NL (nl.f90:21-27)
    int c = IDX(i, j);
    double t1 = (d.UE[c] * 0.5) * (in[c] + in[IDX(i + 1, j)]);
    double t2 = (d.UW[c] * 0.5) * (in[c] + in[IDX(i - 1, j)]);
    double t3 = (d.VN[c] * 0.5) * (in[c] + in[IDX(i, j + 1)]);
    double t4 = (d.VS[c] * 0.5) * (in[c] + in[IDX(i, j - 1)]);
    return ((t1 - t2) + t3) - t4;
}

// Cross-derivative term 0.25*sum(+-K*(diagonal differences)) with K = coefficient
// array evaluated at the four face neighbours (dif_diagonal.f90:13-23 with K=J*Q12;
// iter_u.f90:31-41 with K=J*xix*etx and K=J*xiy*ety).
__device__ __forceinline__ double cross_at(const Dev &d, const double *K, const double *f, int i, int j)
{
    double fne = f[IDX(i + 1, j + 1)], fse = f[IDX(i + 1, j - 1)];
    double fnw = f[IDX(i - 1, j + 1)], fsw = f[IDX(i - 1, j - 1)];
    double t1 = K[IDX(i + 1, j)] * (fne - fse);
    double t2 = K[IDX(i - 1, j)] * (fnw - fsw);
    double t3 = K[IDX(i, j + 1)] * (fne - fnw);
    double t4 = K[IDX(i, j - 1)] * (fse - fsw);
    return 0.25 * (((t1 - t2) + t3) - t4);
}

__device__ __forceinline__ double dif_at(const Dev &d, const double *in, int i, int j)
{   // DIF (dif.f90:13-23)
    int c = IDX(i, j);
    double dd = cross_at(d, d.JQ12, in, i, j);
    double p = in[c];
    double a = d.DE[c] * (in[IDX(i + 1, j)] - p);
    double b = d.DW[c] * (in[IDX(i - 1, j)] - p);
    double e = d.DN[c] * (in[IDX(i, j + 1)] - p);
    double f = d.DS[c] * (in[IDX(i, j - 1)] - p);
    return (((a + b) + e) + f) + dd;
}

__device__ __forceinline__ void psource_at(const Dev &d, int i, int j, double &su, double &sv)
{   // P_SOURCE (p_source.f90:9-27); P ghost values are read as stored
    const double *J = d.DJAC, *P = d.P;
    int e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
    double a = ((((J[e] * d.XIX[e]) * P[e] - (J[w] * d.XIX[w]) * P[w]) + (J[nn] * d.ETX[nn]) * P[nn]) - (J[s] * d.ETX[s]) * P[s]);
    double b = ((((J[e] * d.XIY[e]) * P[e] - (J[w] * d.XIY[w]) * P[w]) + (J[nn] * d.ETY[nn]) * P[nn]) - (J[s] * d.ETY[s]) * P[s]);
    su = -(0.5 * a);
    sv = -(0.5 * b);
}

__device__ __forceinline__ double u1_at(const Dev &d, int c) { return d.XIX[c] * d.U[c] + d.XIY[c] * d.V[c]; }
__device__ __forceinline__ double u2_at(const Dev &d, int c) { return d.ETX[c] * d.U[c] + d.ETY[c] * d.V[c]; }

// Predictor right-hand side of the first AF factor (iter_u.f90:31-46) with the
// wall/far-field folding of BCU (bcu.f90:15, 35).
__device__ __forceinline__ double af_su1_at(const Dev &d, int kind, const double *phi, const double *phin,
                                            const double *nl, const double *nlm1, const double *dif,
                                            const double *src, int i, int j)
{
    int c = IDX(i, j);
    const bool tk = (kind == FVM_FIELD_T);
    const double rek = tk ? d.pe : d.re;
    const double *JDT = tk ? d.PJDT : d.RJDT;
    double s = (JDT[c] * phin[c] - (3.0 * rek) * nl[c]) + rek * nlm1[c];
    s = s + dif[c];
    if (!tk) s = s + (2.0 * rek) * src[c];
    s = s + cross_at(d, d.JXE, phi, i, j);
    const Coef &cf = tk ? d.cTX : d.cUX;
    if (i == 1) {
        double w = (kind == FVM_FIELD_U) ? d.UFW[j] : (kind == FVM_FIELD_V ? d.VFW[j] : d.TFW[j]);
        s = s + (2.0 * cf.awall[j]) * w;
    }
    if (i == d.NI - 1) {
        double f = (kind == FVM_FIELD_U) ? d.FFU[j] : (kind == FVM_FIELD_V ? d.FFV[j] : d.FFT[j]);
        s = s + (2.0 * cf.afar[j]) * f;
    }
    return s;
}

struct FieldRefs {
    double *phi, *phin, *nl, *nlm1, *dif, *src, *su;
    const double *wallF, *farF;
};

__device__ __forceinline__ FieldRefs field_refs(const Dev &d, int kind)
{
    if (kind == FVM_FIELD_U) return {d.U, d.U_N, d.NLX, d.NLX_NM1, d.DIFX, d.S_U, d.SU, d.UFW, d.FFU};
    if (kind == FVM_FIELD_V) return {d.V, d.V_N, d.NLY, d.NLY_NM1, d.DIFY, d.S_V, d.SUV, d.VFW, d.FFV};
    return {d.T, d.T_N, d.ADV, d.ADV_NM1, d.DIFT, nullptr, d.SUT, d.TFW, d.FFT};
}

// ---------------------------------------------------------------------------------
// Elementwise / stencil kernels.  Interior cells are mapped to a 2-D grid with i
// fastest: blockIdx.y = j-1.
// ---------------------------------------------------------------------------------
#define INTERIOR_IJ                                                   \
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1; \
    if (i > d.NI - 1 || j > d.NJ - 1) return;

__global__ void k_begin(Dev d)
{   // Main.f90:52-54 (full arrays)
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.n) return;
    d.U_N[k] = d.U[k];
    d.V_N[k] = d.V[k];
    d.T_N[k] = d.T[k];
}

__global__ void k_farfield_step(Dev d)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > d.NJ - 1) return;
    const int NI = d.NI;
    const double *ph[3] = {d.U_N, d.V_N, d.T_N};
    double fin[3] = {d.uin, d.vin, d.tin};
    double *out[3] = {d.FFU, d.FFV, d.FFT};
    double th = d.THETA[IDX(NI, j)];
    bool inflow = th >= 0.5 * d.pi && th <= 1.5 * d.pi;
    double a = 0.5 * (d.XIX[IDX(NI, j)] + d.XIX[IDX(NI - 1, j)]);
    double b = (0.5 * (d.ETX[IDX(NI, j)] + d.ETX[IDX(NI - 1, j)])) * 0.25;
    for (int f = 0; f < 3; f++) {
        const double *q = ph[f];
        double dq = ((q[IDX(NI, j + 1)] + q[IDX(NI - 1, j + 1)]) - q[IDX(NI, j - 1)]) - q[IDX(NI - 1, j - 1)];
        out[f][j] = inflow ? fin[f]
                           : 0.5 * (q[IDX(NI, j)] + q[IDX(NI - 1, j)]) - (d.dt * d.uin) * (a * (q[IDX(NI, j)] - q[IDX(NI - 1, j)]) + b * dq);
    }
}

// CONTRA_VEL (contra_vel.f90:9-21,125); with_poisson additionally forms the
// Poisson source (1/dt)*div and the first sweep's SU = div/dt - DD(P)
// (iter_p.f90:24-30) and resets the iteration control.
__global__ void k_contra_vel(Dev d, int with_poisson)
{
    INTERIOR_IJ
    const double *J = d.DJAC;
    int c = IDX(i, j), e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
    double ju1 = J[c] * u1_at(d, c), ju2 = J[c] * u2_at(d, c);
    double ue = 0.5 * (ju1 + J[e] * u1_at(d, e));
    double uw = (i == 1) ? 0.0 : 0.5 * (ju1 + J[w] * u1_at(d, w));
    double vn = 0.5 * (ju2 + J[nn] * u2_at(d, nn));
    double vs = 0.5 * (ju2 + J[s] * u2_at(d, s));
    d.UE[c] = ue;
    d.UW[c] = uw;
    d.VN[c] = vn;
    d.VS[c] = vs;
    if (with_poisson) {
        double dv = d.rdt * (((ue - uw) + vn) - vs);
        d.DIVDT[c] = dv;
        d.SU[c] = dv - cross_at(d, d.JQ12, d.P, i, j);
        if (i == 1 && j == 1) {
            d.pctl->niter = 0;
            d.pctl->done = 0;
            d.pctl->capped = 0;
            d.pctl->resip = 0.0;
        }
    }
}

__global__ void k_nl(Dev d, int field)
{
    INTERIOR_IJ
    int c = IDX(i, j);
    FieldRefs f = field_refs(d, field);
    f.nlm1[c] = f.nl[c];
    f.nl[c] = nl_at(d, f.phin, i, j);
}

__global__ void k_dif(Dev d, int field)
{
    INTERIOR_IJ
    FieldRefs f = field_refs(d, field);
    d.DD[IDX(i, j)] = cross_at(d, d.JQ12, f.phin, i, j);
    f.dif[IDX(i, j)] = dif_at(d, f.phin, i, j);
}

__global__ void k_psource(Dev d)
{
    INTERIOR_IJ
    double su, sv;
    psource_at(d, i, j, su, sv);
    d.S_U[IDX(i, j)] = su;
    d.S_V[IDX(i, j)] = sv;
}

// Fused explicit phase of a step (Main.f90:61-74 plus the first-factor right-hand
// sides of ITER_U/ITER_V/ITER_T, which depend only on step-n data).
__global__ void k_explicit(Dev d, int thermal)
{
    INTERIOR_IJ
    int c = IDX(i, j);
    d.NLX_NM1[c] = d.NLX[c];
    d.NLY_NM1[c] = d.NLY[c];
    d.ADV_NM1[c] = d.ADV[c];
    double nlx = nl_at(d, d.U_N, i, j), nly = nl_at(d, d.V_N, i, j);
    d.NLX[c] = nlx;
    d.NLY[c] = nly;
    d.DIFX[c] = dif_at(d, d.U_N, i, j);
    d.DIFY[c] = dif_at(d, d.V_N, i, j);
    double su, sv;
    psource_at(d, i, j, su, sv);
    d.S_U[c] = su;
    d.S_V[c] = sv;
    if (thermal) {
        d.ADV[c] = nl_at(d, d.T_N, i, j);
        d.DIFT[c] = dif_at(d, d.T_N, i, j);
    }
    d.SU[c] = af_su1_at(d, FVM_FIELD_U, d.U_N, d.U_N, d.NLX, d.NLX_NM1, d.DIFX, d.S_U, i, j);
    d.SUV[c] = af_su1_at(d, FVM_FIELD_V, d.V_N, d.V_N, d.NLY, d.NLY_NM1, d.DIFY, d.S_V, i, j);
    if (thermal) d.SUT[c] = af_su1_at(d, FVM_FIELD_T, d.T_N, d.T_N, d.ADV, d.ADV_NM1, d.DIFT, nullptr, i, j);
}

__global__ void k_af_su1(Dev d, int field)
{
    INTERIOR_IJ
    FieldRefs f = field_refs(d, field);
    f.su[IDX(i, j)] = af_su1_at(d, field, f.phi, f.phin, f.nl, f.nlm1, f.dif, f.src, i, j);
}

// Second-factor right-hand side (iter_u.f90:86-99, iter_T.f90:86-98) with the
// BCU folding; cross term from xfield (V for ITER_T when the reference's V is kept).
__global__ void k_af_su2(Dev d, int field, const double *xfield)
{
    INTERIOR_IJ
    int c = IDX(i, j);
    FieldRefs f = field_refs(d, field);
    const bool tk = field == FVM_FIELD_T;
    const double *JDT = tk ? d.PJDT : d.RJDT;
    double s = JDT[c] * f.phi[c] + cross_at(d, d.JYE, xfield, i, j);
    const Coef &cf = tk ? d.cTY : d.cUY;
    if (i == 1) s = s + (2.0 * cf.awall[j]) * f.wallF[j];
    if (i == d.NI - 1) s = s + (2.0 * cf.afar[j]) * f.farF[j];
    f.su[c] = s;
}

// u^ = u* -/+ dt S/J on the interior (Main.f90:80-84, 99-103) with the BCU/BCV ghost
// refresh of the updated cells.  with_psource recomputes S from P first and derives
// the P ghosts of BCP (bcp.f90:19-30,36-42) from the interior as well.
__global__ void k_grad(Dev d, double sign, int with_psource)
{
    INTERIOR_IJ
    int c = IDX(i, j);
    double su, sv;
    if (with_psource) {
        // P_SOURCE with BCP ghost values taken from the interior (identical to the
        // stored ghosts after BCP).
        const double *J = d.DJAC;
        double *P = d.P;
        const int NI = d.NI;
        int e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, jwrap(d, j + 1)), s = IDX(i, jwrap(d, j - 1));
        double pe = P[e], pw = P[w];
        if (i == 1) pw = P[IDX(1, j)];
        if (i == NI - 1) pe = (3.0 * P[IDX(NI - 1, j)] - 3.0 * P[IDX(NI - 2, j)]) + P[IDX(NI - 3, j)];
        int ge = IDX(i + 1, j), gw = IDX(i - 1, j), gn = IDX(i, j + 1), gs = IDX(i, j - 1);
        double a = ((((J[ge] * d.XIX[ge]) * pe - (J[gw] * d.XIX[gw]) * pw) + (J[gn] * d.ETX[gn]) * P[nn]) - (J[gs] * d.ETX[gs]) * P[s]);
        double b = ((((J[ge] * d.XIY[ge]) * pe - (J[gw] * d.XIY[gw]) * pw) + (J[gn] * d.ETY[gn]) * P[nn]) - (J[gs] * d.ETY[gs]) * P[s]);
        su = -(0.5 * a);
        sv = -(0.5 * b);
        d.S_U[c] = su;
        d.S_V[c] = sv;
        // BCP ghosts derived from this interior cell
        if (i == 1) {
            double g = P[c];
            P[IDX(0, j)] = g;
            if (j == 1) P[IDX(0, d.NJ)] = g;
            if (j == d.NJ - 1) P[IDX(0, 0)] = g;
        }
        if (i == NI - 1) {
            double g = (3.0 * P[IDX(NI - 1, j)] - 3.0 * P[IDX(NI - 2, j)]) + P[IDX(NI - 3, j)];
            P[IDX(NI, j)] = g;
            if (j == 1) P[IDX(NI, d.NJ)] = g;
            if (j == d.NJ - 1) P[IDX(NI, 0)] = g;
        }
        if (j == 1) P[IDX(i, d.NJ)] = P[c];
        if (j == d.NJ - 1) P[IDX(i, 0)] = P[c];
    } else {
        su = d.S_U[c];
        sv = d.S_V[c];
    }
    double du = (su * d.dt) / d.DJAC[c], dv = (sv * d.dt) / d.DJAC[c];
    double u = sign < 0 ? d.U[c] - du : d.U[c] + du;
    double v = sign < 0 ? d.V[c] - dv : d.V[c] + dv;
    d.U[c] = u;
    d.V[c] = v;
    ghost_dirichlet(d, d.U, i, j, u, d.UFW, d.FFU);
    ghost_dirichlet(d, d.V, i, j, v, d.VFW, d.FFV);
}

// BCP ghost refresh from the interior (bcp.f90:19-30, 36-42) over every ghost cell.
__global__ void k_bcp_ghosts(Dev d)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int NI = d.NI, NJ = d.NJ;
    double *P = d.P;
    auto cubic = [&](int j) { return (3.0 * P[IDX(NI - 1, j)] - 3.0 * P[IDX(NI - 2, j)]) + P[IDX(NI - 3, j)]; };
    if (t >= 1 && t <= NJ - 1) {
        P[IDX(0, t)] = P[IDX(1, t)];
        P[IDX(NI, t)] = cubic(t);
    }
    if (t <= NI) {
        int i = t;
        double r0, rn;
        if (i == 0) { r0 = P[IDX(1, NJ - 1)]; rn = P[IDX(1, 1)]; }
        else if (i == NI) { r0 = cubic(NJ - 1); rn = cubic(1); }
        else { r0 = P[IDX(i, NJ - 1)]; rn = P[IDX(i, 1)]; }
        P[IDX(i, 0)] = r0;
        P[IDX(i, NJ)] = rn;
    }
}

// ---------------------------------------------------------------------------------
// Line sweeps (warp per line)
// ---------------------------------------------------------------------------------
enum { BCK_DIRICHLET = 0, BCK_POISSON = 1 };

// Ghost values of radial row j taken from its current interior (the BC call that
// precedes the sweep in the reference: BCU before iter_u.f90:50, BCP before
// iter_p.f90:34).  Writes phi(0,j), phi(NI,j) and, for j = 1 / NJ-1, the
// branch-cut row with its corners.
template <int BCK>
__device__ void refresh_row_ghosts(const Dev &d, double *phi, int j, const double *wallF, const double *farF, int lane)
{
    const int NI = d.NI, NJ = d.NJ;
    double g0, gn;
    if (BCK == BCK_POISSON) {
        g0 = phi[IDX(1, j)];
        gn = (3.0 * phi[IDX(NI - 1, j)] - 3.0 * phi[IDX(NI - 2, j)]) + phi[IDX(NI - 3, j)];
    } else {
        g0 = (-phi[IDX(1, j)]) + 2.0 * wallF[j];
        gn = (-phi[IDX(NI - 1, j)]) + 2.0 * farF[j];
    }
    int rowdst = (j == 1) ? NJ : ((j == NJ - 1) ? 0 : -1);
    if (rowdst >= 0) {
        for (int i = 1 + lane; i <= NI - 1; i += WARP) phi[IDX(i, rowdst)] = phi[IDX(i, j)];
    }
    if (lane == 0) {
        phi[IDX(0, j)] = g0;
        phi[IDX(NI, j)] = gn;
        if (rowdst >= 0) {
            phi[IDX(0, rowdst)] = g0;
            phi[IDX(NI, rowdst)] = gn;
        }
    }
}

// Zebra radial-line sweep: lines j of one colour (colour 0: odd j) solve
//   -AW x(i-1) + AP x(i) - AE x(i+1) = AN phi(i,j+1) + AS phi(i,j-1) + SU
// with the neighbour rows read through periodic wrap (lisolv.f90:72-84,
// iter_u.f90:52-64).  Colour 0 first refreshes the ghosts of its own row and of the
// next (even) row from the pre-sweep values.
template <int M, int BCK>
__global__ void __launch_bounds__(128) k_radial(Dev d, LineSys s, Coef cf, const double *SU, double *phi, int colour,
                                                int refresh, const double *wallF, const double *farF, int early_exit)
{
    if (early_exit && d.pctl->done) return;
    const int lane = threadIdx.x & (WARP - 1);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) / WARP;
    const int half = (d.NJ - 1) / 2;
    if (w >= half) return;
    const int j = 2 * w + 1 + colour;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const int n = s.n;
    if (refresh) {
        refresh_row_ghosts<BCK>(d, phi, j, wallF, farF, lane);
        if (j + 1 <= d.NJ - 1) refresh_row_ghosts<BCK>(d, phi, j + 1, wallF, farF, lane);
        __syncwarp();
    }
    double v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        v[k] = 0.0;
        if (e < n) {
            int c = IDX(e + 1, j);
            v[k] = (cf.AN[c] * phi[IDX(e + 1, jn)] + cf.AS[c] * phi[IDX(e + 1, js)]) + SU[c];
        }
    }
    const size_t base = size_t(j - 1) * WARP * M;
    line_apply<double, M>(v, s.invD + base, s.fa + base, s.fb + base, lane);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        if (e < n) phi[IDX(e + 1, j)] = v[k];
    }
}

// Zebra circumferential-line sweep of the predictor's second factor: lines i of one
// colour (colour 0: odd i) solve the cyclic system
//   -AS x(j-1) + AP x(j) - AN x(j+1) = AE phi(i+1,j) + AW phi(i-1,j) + SU
// (iter_u.f90:104-119 with the periodic coupling made implicit).  ghosts != 0 also
// writes the BCT/BCU ghost cells derived from the new values.
template <int M>
__global__ void __launch_bounds__(128) k_theta(Dev d, LineSys s, Coef cf, const double *SU, double *phi, int colour,
                                               int ghosts, const double *wallF, const double *farF)
{
    const int lane = threadIdx.x & (WARP - 1);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) / WARP;
    const int i = 2 * w + 1 + colour;
    if (i > d.NI - 1) return;
    const int n = s.n;
    double v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        v[k] = 0.0;
        if (e < n) {
            int c = IDX(i, e + 1);
            v[k] = (cf.AE[c] * phi[IDX(i + 1, e + 1)] + cf.AW[c] * phi[IDX(i - 1, e + 1)]) + SU[c];
        }
    }
    const size_t base = size_t(i - 1) * WARP * M;
    line_apply<double, M>(v, s.invD + base, s.fa + base, s.fb + base, lane);
    line_cyclic_fix<double, M>(v, s.z + base, s.cv[i - 1], s.sinv[i - 1], n, lane);
    __syncwarp();
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        if (e < n) {
            phi[IDX(i, e + 1)] = v[k];
            if (ghosts) ghost_dirichlet(d, phi, i, e + 1, v[k], wallF, farF);
        }
    }
}

// ---------------------------------------------------------------------------------
// Poisson residual (iter_p.f90:37-51) fused with the next sweep's lagged cross term
// (iter_p.f90:24-30).  Deterministic two-level reduction; the last block decides
// convergence and publishes the iteration count.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void block_sum2(double &a, double &b, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int wid = threadIdx.x / WARP, lane = threadIdx.x & 31, nw = blockDim.x / WARP;
    __syncthreads();
    if (lane == 0) { sh[2 * wid] = a; sh[2 * wid + 1] = b; }
    __syncthreads();
    if (wid == 0) {
        a = lane < nw ? sh[2 * lane] : 0.0;
        b = lane < nw ? sh[2 * lane + 1] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
    }
}

__global__ void __launch_bounds__(256) k_pres(Dev d)
{
    __shared__ double sh[64];
    __shared__ bool last;
    if (d.pctl->done) return;
    const int it = d.pctl->niter + 1;
    const bool check = (it % d.res_every == 0) || (it >= d.nswpp);
    const int NI = d.NI, ni1 = NI - 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double ra = 0.0, pa = 0.0;
    if (e < ni1 * (d.NJ - 1)) {
        const int i = e % ni1 + 1, j = e / ni1 + 1;
        const int c = IDX(i, j);
        const double *P = d.P;
        if (check) {
            const Coef &cf = d.cP;
            double p = P[c];
            double r = ((((cf.AE[c] * P[IDX(i + 1, j)] + cf.AW[c] * P[IDX(i - 1, j)]) + cf.AN[c] * P[IDX(i, jwrap(d, j + 1))])
                         + cf.AS[c] * P[IDX(i, jwrap(d, j - 1))]) + d.SU[c]) - cf.AP[c] * p;
            ra = fabs(r);
            pa = fabs(cf.AP[c] * p);
        }
        d.SU[c] = d.DIVDT[c] - cross_at(d, d.JQ12, P, i, j);
    }
    block_sum2(ra, pa, sh);
    if (threadIdx.x == 0) {
        d.partial[2 * blockIdx.x] = ra;
        d.partial[2 * blockIdx.x + 1] = pa;
        __threadfence();
        unsigned t = atomicInc(&d.pctl->ticket, gridDim.x - 1);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
        a += ((volatile double *)d.partial)[2 * k];
        b += ((volatile double *)d.partial)[2 * k + 1];
    }
    block_sum2(a, b, sh);
    if (threadIdx.x == 0) {
        d.pctl->niter = it;
        if (check) {
            double resip = a / b;
            d.pctl->resip = resip;
            if (!(resip > d.resimax && it < d.nswpp)) {
                d.pctl->done = 1;
                d.pctl->capped = (resip > d.resimax) ? 1 : 0;
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// CALCCOEF (calccoef.f90:9-120): per-j wall contributions, CFL maximum, then a
// single-thread fixed-order sum (the reference's J order).
// ---------------------------------------------------------------------------------
__global__ void k_calc_rows(Dev d)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > d.NJ - 1) return;
    const int c = IDX(1, j);
    const double X = d.X[c], Y = d.Y[c];
    const double xa = d.XG[IDX(1, j)], ya = d.YG[IDX(1, j)], xb = d.XG[IDX(1, j + 1)], yb = d.YG[IDX(1, j + 1)];
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
    double TH2 = atan((Y - Y1) / (X - X1));
    double sg = asin((Y - Y1) / DN2);
    if (TH2 >= 0.0 && sg > 0.0) TH2 = TH2;
    else if (TH2 < 0.0 && sg > 0.0) TH2 = d.pi + TH2;
    else if (TH2 >= 0.0 && sg <= 0.0) TH2 = d.pi + TH2;
    else if (TH2 < 0.0 && sg < 0.0) TH2 = 2.0 * d.pi + TH2;
    double dudn = ((d.U[c] * sin(TH2) - d.V[c] * cos(TH2)) - d.vel_rot) / DN1;
    double dtdn = (d.T[c] - d.t_wall) / DN1;
    double th = d.THETA[c], ar = d.AREA[c], p = d.P[c];
    double *row = d.coefrow + 8 * j;
    row[0] = ((2.0 * p) * ar) * cos(th);
    row[1] = ((2.0 * p) * ar) * sin(th);
    row[2] = (((2.0 / d.re) * dudn) * ar) * sin(th);
    row[3] = (((2.0 / d.re) * dudn) * ar) * cos(th);
    row[4] = dtdn * ar;
}

__global__ void k_cfl(Dev d)
{
    INTERIOR_IJ
    int c = IDX(i, j);
    double l = d.dt * (fabs(d.XIX[c] * d.U[c] + d.XIY[c] * d.V[c]) + fabs(d.ETX[c] * d.U[c] + d.ETY[c] * d.V[c]));
    atomicMax(d.cflbits, (unsigned long long)__double_as_longlong(l));
}

__global__ void k_calc_final(Dev d, double rtime, fvm_coeffs *out)
{
    double pd = 0.0, pl = 0.0, td = 0.0, tl = 0.0, nu = 0.0;
    for (int j = 1; j <= d.NJ - 1; j++) {
        const double *row = d.coefrow + 8 * j;
        pd = pd - row[0];
        pl = pl - row[1];
        td = td + row[2];
        tl = tl - row[3];
        nu = nu + row[4];
    }
    const double *P = d.P;
    double pg11 = 0.25 * (((P[IDX(1, 1)] + P[IDX(1, 0)]) + P[IDX(0, 1)]) + P[IDX(0, 0)]);
    out->time = rtime;
    out->cfl = __longlong_as_double((long long)*d.cflbits);
    out->cpb = 2.0 * (0.0 - pg11);   // far-field node value never assigned: zero (calccoef.f90:41-45)
    out->cd_p = pd;
    out->cl_p = pl;
    out->cd_v = td;
    out->cl_v = tl;
    out->cd = pd + td;
    out->cl = pl + tl;
    out->nu = -nu / d.scal[0];
    out->sweeps = d.pctl->niter;
    out->resid = d.pctl->resip;
    *d.cflbits = 0ull;
}

// ---------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------
namespace {

inline dim3 interior_grid(const fvm_ctx *c) { return dim3((c->NI - 1 + 127) / 128, c->NJ - 1); }

template <int BCK>
int launch_radial(fvm_ctx *c, const LineSys &s, const Coef &cf, const double *SU, double *phi, int colour,
                  int refresh, const double *wallF, const double *farF, int early_exit)
{
    const int half = (c->NJ - 1) / 2;
    const int blocks = (half * WARP + 127) / 128;
    const Dev &d = c->d;
    switch (s.M) {
#define CASE(MM)                                                                                   \
    case MM:                                                                                       \
        k_radial<MM, BCK><<<blocks, 128, 0, c->stream>>>(d, s, cf, SU, phi, colour, refresh, wallF, farF, early_exit); \
        break;
        CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8)
        CASE(9) CASE(10) CASE(11) CASE(12) CASE(13) CASE(14) CASE(15) CASE(16)
#undef CASE
    default:
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int launch_theta(fvm_ctx *c, const LineSys &s, const Coef &cf, const double *SU, double *phi, int colour,
                 int ghosts, const double *wallF, const double *farF)
{
    const int nl = (c->NI - 1 + 1 - colour) / 2;
    const int blocks = (nl * WARP + 127) / 128;
    const Dev &d = c->d;
    switch (s.M) {
#define CASE(MM)                                                                                   \
    case MM:                                                                                       \
        k_theta<MM><<<blocks, 128, 0, c->stream>>>(d, s, cf, SU, phi, colour, ghosts, wallF, farF); \
        break;
        CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8)
        CASE(9) CASE(10) CASE(11) CASE(12) CASE(13) CASE(14) CASE(15) CASE(16)
#undef CASE
    default:
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

#define RC(x)                 \
    do {                      \
        int rc_ = (x);        \
        if (rc_) return rc_;  \
    } while (0)

// The predictor of one field after its first-factor SU is in place.
int predictor_sweeps(fvm_ctx *c, int field)
{
    Dev &d = c->d;
    const bool tk = field == FVM_FIELD_T;
    const LineSys &sx = tk ? d.sTX : d.sUX;
    const LineSys &sy = tk ? d.sTY : d.sUY;
    const Coef &cx = tk ? d.cTX : d.cUX;
    const Coef &cy = tk ? d.cTY : d.cUY;
    double *phi = field == FVM_FIELD_U ? d.U : (field == FVM_FIELD_V ? d.V : d.T);
    double *su = field == FVM_FIELD_U ? d.SU : (field == FVM_FIELD_V ? d.SUV : d.SUT);
    const double *wf = field == FVM_FIELD_U ? d.UFW : (field == FVM_FIELD_V ? d.VFW : d.TFW);
    const double *farF = field == FVM_FIELD_U ? d.FFU : (field == FVM_FIELD_V ? d.FFV : d.FFT);
    // sweep 1 (radial lines), ghosts refreshed from the pre-sweep field (BCU)
    RC(launch_radial<BCK_DIRICHLET>(c, sx, cx, su, phi, 0, 1, wf, farF, 0));
    RC(launch_radial<BCK_DIRICHLET>(c, sx, cx, su, phi, 1, 0, wf, farF, 0));
    // second factor right-hand side from the first-sweep field
    const double *xf = (tk && c->p.iter_t_bug) ? d.V : phi;
    k_af_su2<<<interior_grid(c), 128, 0, c->stream>>>(d, field, xf);
    FVM_LAUNCH_CHECK(c);
    RC(launch_theta(c, sy, cy, su, phi, 0, tk ? 1 : 0, wf, farF));
    RC(launch_theta(c, sy, cy, su, phi, 1, tk ? 1 : 0, wf, farF));
    return FVM_OK;
}

}  // namespace

int run_begin_step(fvm_ctx *c)
{
    Dev &d = c->d;
    c->rtime = c->rtime + c->p.dt;
    c->niter_time += 1;
    k_begin<<<(c->n + 255) / 256, 256, 0, c->stream>>>(d);
    k_farfield_step<<<(c->NJ + 127) / 128, 128, 0, c->stream>>>(d);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_contra_vel(fvm_ctx *c)
{
    k_contra_vel<<<interior_grid(c), 128, 0, c->stream>>>(c->d, 0);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_nl(fvm_ctx *c, int field)
{
    k_nl<<<interior_grid(c), 128, 0, c->stream>>>(c->d, field);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_dif(fvm_ctx *c, int field)
{
    k_dif<<<interior_grid(c), 128, 0, c->stream>>>(c->d, field);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_p_source(fvm_ctx *c)
{
    k_psource<<<interior_grid(c), 128, 0, c->stream>>>(c->d);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_iter_u(fvm_ctx *c, int field)
{
    k_af_su1<<<interior_grid(c), 128, 0, c->stream>>>(c->d, field);
    FVM_LAUNCH_CHECK(c);
    return predictor_sweeps(c, field);
}

int run_remove_grad(fvm_ctx *c)
{
    k_grad<<<interior_grid(c), 128, 0, c->stream>>>(c->d, -1.0, 0);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

static int poisson_graph(fvm_ctx *c, int batch)
{
    if (c->pgraph && c->pgraph_batch == batch) return FVM_OK;
    if (c->pgraph) {
        cudaGraphExecDestroy(c->pgraph);
        c->pgraph = nullptr;
    }
    Dev &d = c->d;
    cudaGraph_t g = nullptr;
    FVM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = FVM_OK;
    for (int b = 0; b < batch && rc == FVM_OK; b++) {
        rc = launch_radial<BCK_POISSON>(c, d.sP, d.cP, d.SU, d.P, 0, 1, nullptr, nullptr, 1);
        if (rc == FVM_OK) rc = launch_radial<BCK_POISSON>(c, d.sP, d.cP, d.SU, d.P, 1, 0, nullptr, nullptr, 1);
        if (rc == FVM_OK) k_pres<<<c->nblk_res, 256, 0, c->stream>>>(d);
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) {
        c->err = std::string("Poisson graph capture: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&c->pgraph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->err = std::string("Poisson graph instantiate: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    c->pgraph_batch = batch;
    return FVM_OK;
}

int run_iter_p(fvm_ctx *c, double *resid, int *sweeps)
{
    Dev &d = c->d;
    k_contra_vel<<<interior_grid(c), 128, 0, c->stream>>>(d, 1);
    FVM_LAUNCH_CHECK(c);
    const int batch = 16;
    RC(poisson_graph(c, batch));
    int status = FVM_OK;
    // The device stops itself at the cap; the host bound only guards against a
    // control block that never reports completion.
    const long max_launches = (long)c->p.nswpp / batch + 2;
    for (long launch = 0;; launch++) {
        if (launch >= max_launches) {
            c->err = "Poisson iteration did not report completion within the sweep cap";
            return FVM_ERR_TIMEOUT;
        }
        FVM_CUDA(c, cudaGraphLaunch(c->pgraph, c->stream));
        FVM_CUDA(c, cudaMemcpyAsync(c->h_pctl, d.pctl, sizeof(PCtl), cudaMemcpyDeviceToHost, c->stream));
        FVM_CUDA(c, cudaStreamSynchronize(c->stream));
        if (c->h_pctl->done) break;
    }
    if (c->h_pctl->capped) status = FVM_ERR_NOCONV;
    if (!std::isfinite(c->h_pctl->resip)) {
        c->err = "non-finite Poisson residual";
        status = FVM_ERR_NAN;
    }
    if (resid) *resid = c->h_pctl->resip;
    if (sweeps) *sweeps = c->h_pctl->niter;
    k_bcp_ghosts<<<(c->NI + c->NJ + 127) / 128, 128, 0, c->stream>>>(d);
    FVM_LAUNCH_CHECK(c);
    return status;
}

int run_correct(fvm_ctx *c)
{
    k_grad<<<interior_grid(c), 128, 0, c->stream>>>(c->d, +1.0, 1);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_iter_t(fvm_ctx *c)
{
    k_af_su1<<<interior_grid(c), 128, 0, c->stream>>>(c->d, FVM_FIELD_T);
    FVM_LAUNCH_CHECK(c);
    return predictor_sweeps(c, FVM_FIELD_T);
}

int run_calccoef(fvm_ctx *c, fvm_coeffs *out)
{
    Dev &d = c->d;
    k_calc_rows<<<(c->NJ + 127) / 128, 128, 0, c->stream>>>(d);
    k_cfl<<<interior_grid(c), 128, 0, c->stream>>>(d);
    fvm_coeffs *dout = reinterpret_cast<fvm_coeffs *>(d.scal + 4);
    static_assert(sizeof(fvm_coeffs) <= 12 * sizeof(double), "coeff scratch");
    k_calc_final<<<1, 1, 0, c->stream>>>(d, c->rtime, dout);
    FVM_LAUNCH_CHECK(c);
    FVM_CUDA(c, cudaMemcpyAsync(&c->last, dout, sizeof(fvm_coeffs), cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (out) *out = c->last;
    if (!std::isfinite(c->last.cd) || !std::isfinite(c->last.cl)) {
        c->err = "non-finite drag or lift";
        return FVM_ERR_NAN;
    }
    return FVM_OK;
}

int run_step(fvm_ctx *c, int nsteps, fvm_coeffs *out)
{
    Dev &d = c->d;
    int status = FVM_OK;
    c->hist.clear();
    for (int s = 0; s < nsteps; s++) {
        RC(run_begin_step(c));
        k_contra_vel<<<interior_grid(c), 128, 0, c->stream>>>(d, 0);
        k_explicit<<<interior_grid(c), 128, 0, c->stream>>>(d, c->p.thermal);
        FVM_LAUNCH_CHECK(c);
        RC(predictor_sweeps(c, FVM_FIELD_U));
        RC(predictor_sweeps(c, FVM_FIELD_V));
        RC(run_remove_grad(c));
        int rc = run_iter_p(c, nullptr, nullptr);
        if (rc == FVM_ERR_NOCONV) status = FVM_ERR_NOCONV;
        else if (rc) return rc;
        RC(run_correct(c));
        if (c->p.thermal) RC(predictor_sweeps(c, FVM_FIELD_T));
        fvm_coeffs co;
        RC(run_calccoef(c, &co));
        c->hist.push_back(co);
        if (out) *out = co;
    }
    return status;
}

}  // namespace fvm
