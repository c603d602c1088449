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
#include "fvm_ops.cuh"

namespace fvm {

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
// Poisson source (1/dt)*div (iter_p.f90:27-29) and resets the iteration control.
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
        d.DIVDT[c] = d.rdt * (((ue - uw) + vn) - vs);
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
// Zebra radial-line sweep: lines j of one colour (colour 0: odd j) solve
//   -AW x(i-1) + AP x(i) - AE x(i+1) = AN phi(i,j+1) + AS phi(i,j-1) + SU
// with the neighbour rows read through periodic wrap (iter_u.f90:52-64).
// Colour 0 first refreshes the ghosts of its own row and of the next (even) row
// from the pre-sweep values (the BCU call at iter_u.f90:48).
template <int M, int NW, int BCK>
__global__ void __launch_bounds__(128) k_radial(Dev d, LineSys s, Coef cf, const double *SU, double *phi, int colour,
                                                int refresh, const double *wallF, const double *farF)
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
    if (active && refresh && t < WARP) {
        refresh_row_ghosts<BCK>(d, phi, phi, j, wallF, farF, t);
        if (j + 1 <= d.NJ - 1) refresh_row_ghosts<BCK>(d, phi, phi, j + 1, wallF, farF, t);
    }
    double v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        v[k] = 0.0;
        if (active && e < n) {
            int c = IDX(e + 1, j);
            v[k] = (cf.AN[c] * phi[IDX(e + 1, jn)] + cf.AS[c] * phi[IDX(e + 1, js)]) + SU[c];
        }
    }
    to_chunks<double, M, NW>(v, sm[gib], t);
    const size_t base = size_t(j - 1) * TG * M;
    group_apply<double, M, NW>(v, s.invD + base, s.fa + base, s.fb + base, t, xch[gib]);
    to_interleaved<double, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) phi[IDX(e + 1, j)] = v[k];
    }
}

// Zebra circumferential-line sweep of the predictor's second factor: lines i of one
// colour (colour 0: odd i) solve the cyclic system
//   -AS x(j-1) + AP x(j) - AN x(j+1) = AE phi(i+1,j) + AW phi(i-1,j) + SU
// (iter_u.f90:104-119 with the periodic coupling made implicit).  ghosts != 0 also
// writes the BCT/BCU ghost cells derived from the new values.
template <int M, int NW>
__global__ void __launch_bounds__(128) k_theta(Dev d, LineSys s, Coef cf, const double *SU, double *phi, int colour,
                                               int ghosts, const double *wallF, const double *farF)
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
        v[k] = 0.0;
        if (active && e < n) {
            int c = IDX(i, e + 1);
            v[k] = (cf.AE[c] * phi[IDX(i + 1, e + 1)] + cf.AW[c] * phi[IDX(i - 1, e + 1)]) + SU[c];
        }
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
            phi[IDX(i, e + 1)] = v[k];
            if (ghosts) ghost_dirichlet(d, phi, i, e + 1, v[k], wallF, farF);
        }
    }
}

// ---------------------------------------------------------------------------------
// FP64 pressure Poisson (iter_p.f90:22-51, lisolv.f90:18-33, bcp.f90:8-42).
// One outer iteration = lagged cross term DD from the iteration's input, BCP ghost
// refresh from that input, a zebra line sweep, and (every res_every-th iteration)
// the scaled-L1 residual.  The sweep reads its input P^(n-1) from Pin and writes
// P^n to Pout (two alternating buffers): colour 0 (odd rows) reads its neighbour
// rows from Pin, colour 1 (even rows) from Pout, exactly the in-place zebra order,
// while DD of both colours still sees P^(n-1) as the reference's lagged term does.
// ---------------------------------------------------------------------------------
template <int M, int NW>
__global__ void __launch_bounds__(128) k_pois64(Dev d, const double *Pin, double *Pout, int colour, int check_done)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sm[G][TG * M + M * NW + 1];
    __shared__ double xch[G][2 * NW];
    int gl, t, gib;
    group_of<NW>(gl, t, gib);
    const bool active = gl < (d.NJ - 1) / 2;
    const int j = active ? 2 * gl + 1 + colour : 1;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const LineSys &s = d.sP;
    const Coef &cf = d.cP;
    const int n = s.n;
    // constants first (factors, couplings, the step's source term)
    const size_t base = size_t(j - 1) * TG * M;
    double fi[M], fa[M], fb[M], an[M], as[M], dv[M];
    load_factors<double, M, NW>(fi, fa, fb, s.invD + base, s.fa + base, s.fb + base, t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        bool ok = active && e < n;
        int c = IDX(e + 1, j);
        an[k] = ok ? cf.AN[c] : 0.0;
        as[k] = ok ? cf.AS[c] : 0.0;
        dv[k] = ok ? d.DIVDT[c] : 0.0;
    }
    griddep_wait();
    if (check_done && d.pctl->done) return;
    if (active && colour == 0 && t < WARP) {   // BCP of this iteration: ghosts of P^(n-1), stored with P^n
        refresh_row_ghosts<BCK_POISSON>(d, Pin, Pout, j, nullptr, nullptr, t);
        if (j + 1 <= d.NJ - 1) refresh_row_ghosts<BCK_POISSON>(d, Pin, Pout, j + 1, nullptr, nullptr, t);
    }
    const double *Pnb = colour ? Pout : Pin;
    double v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        v[k] = 0.0;
        if (active && e < n) {
            int i = e + 1;
            double su = dv[k] - dd_src(d, Pin, i, j);
            v[k] = (an[k] * Pnb[IDX(i, jn)] + as[k] * Pnb[IDX(i, js)]) + su;
        }
    }
    griddep_launch();   // the next kernel may start its constant prologue now
    to_chunks<double, M, NW>(v, sm[gib], t);
    group_apply_r<double, M, NW>(v, fi, fa, fb, t, xch[gib]);
    to_interleaved<double, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) Pout[IDX(e + 1, j)] = v[k];
    }
}

// Residual after an even number of iterations: P^n in P, P^(n-1) in P2.  SU of the
// last sweep is rebuilt from P^(n-1) (with its stored ghosts).  The last block
// publishes the count and decides convergence (iter_p.f90:50-51); inside the
// device-side loop it also ends the loop (cond != 0).
template <int HAS_COND>
__global__ void __launch_bounds__(256) k_pres64(Dev d, cudaGraphConditionalHandle cond)
{
    __shared__ double sh[64];
    __shared__ bool last;
    griddep_wait();
    if (d.pctl->done) return;
    const int it = d.pctl->niter + d.res_every;
    const int ni1 = d.NI - 1, total = ni1 * (d.NJ - 1);
    double ra = 0.0, pa = 0.0;
#pragma unroll
    for (int q = 0; q < RES_CELLS; q++) {
        int e = (blockIdx.x * RES_CELLS + q) * 256 + threadIdx.x;
        if (e < total) {
            int i = e % ni1 + 1, j = e / ni1 + 1, c = IDX(i, j);
            double su = d.DIVDT[c] - dd_src(d, d.P2, i, j);
            double r = pres_at(d, d.P, su, i, j);
            ra += fabs(r);
            pa += fabs(d.cP.AP[c] * d.P[c]);
        }
    }
    griddep_launch();
    if (!grid_sum2(d, ra, pa, sh, last)) return;
    if (threadIdx.x == 0) {
        double resip = ra / pa;
        d.pctl->niter = it;
        d.pctl->resip = resip;
        if (!(resip > d.resimax && it < d.nswpp)) {
            d.pctl->done = 1;
            d.pctl->capped = (resip > d.resimax) ? 1 : 0;
            if (HAS_COND) cudaGraphSetConditional(cond, 0);
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
                  int refresh, const double *wallF, const double *farF, int /*unused*/)
{
    const Dev &d = c->d;
    const int blocks = line_blocks((c->NJ - 1) / 2, s.NW);
    bool ok = dispatch_line(s, [&](auto m, auto nw) {
        k_radial<decltype(m)::value, decltype(nw)::value, BCK>
            <<<blocks, 128, 0, c->stream>>>(d, s, cf, SU, phi, colour, refresh, wallF, farF);
    });
    if (!ok) {
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int launch_theta(fvm_ctx *c, const LineSys &s, const Coef &cf, const double *SU, double *phi, int colour,
                 int ghosts, const double *wallF, const double *farF)
{
    const Dev &d = c->d;
    const int blocks = line_blocks((c->NI - 1 + 1 - colour) / 2, s.NW);
    bool ok = dispatch_line(s, [&](auto m, auto nw) {
        k_theta<decltype(m)::value, decltype(nw)::value>
            <<<blocks, 128, 0, c->stream>>>(d, s, cf, SU, phi, colour, ghosts, wallF, farF);
    });
    if (!ok) {
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    KCOUNT(c);
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
    const bool mixed = c->p.precision == FVM_MIXED;
    // sweep 1 (radial lines), ghosts refreshed from the pre-sweep field (BCU)
    for (int colour = 0; colour < 2; colour++) {
        if (mixed) RC(mixed_predictor_radial(c, sx, cx, su, phi, colour, colour == 0, wf, farF));
        else RC(launch_radial<BCK_DIRICHLET>(c, sx, cx, su, phi, colour, colour == 0, wf, farF, 0));
    }
    // second factor right-hand side from the first-sweep field
    const double *xf = (tk && c->p.iter_t_bug) ? d.V : phi;
    k_af_su2<<<interior_grid(c), 128, 0, c->stream>>>(d, field, xf);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    for (int colour = 0; colour < 2; colour++) {
        if (mixed) RC(mixed_predictor_theta(c, sy, cy, su, phi, colour, tk ? 1 : 0, wf, farF));
        else RC(launch_theta(c, sy, cy, su, phi, colour, tk ? 1 : 0, wf, farF));
    }
    return FVM_OK;
}

}  // namespace

int run_begin_step(fvm_ctx *c)
{
    Dev &d = c->d;
    c->rtime = c->rtime + c->p.dt;
    c->niter_time += 1;
    k_begin<<<(c->n + 255) / 256, 256, 0, c->stream>>>(d);
    KCOUNT(c);
    k_farfield_step<<<(c->NJ + 127) / 128, 128, 0, c->stream>>>(d);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_contra_vel(fvm_ctx *c)
{
    k_contra_vel<<<interior_grid(c), 128, 0, c->stream>>>(c->d, 0);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_nl(fvm_ctx *c, int field)
{
    k_nl<<<interior_grid(c), 128, 0, c->stream>>>(c->d, field);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_dif(fvm_ctx *c, int field)
{
    k_dif<<<interior_grid(c), 128, 0, c->stream>>>(c->d, field);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_p_source(fvm_ctx *c)
{
    k_psource<<<interior_grid(c), 128, 0, c->stream>>>(c->d);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_iter_u(fvm_ctx *c, int field)
{
    k_af_su1<<<interior_grid(c), 128, 0, c->stream>>>(c->d, field);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return predictor_sweeps(c, field);
}

int run_remove_grad(fvm_ctx *c)
{
    k_grad<<<interior_grid(c), 128, 0, c->stream>>>(c->d, -1.0, 0);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int launch_pois64(fvm_ctx *c, const double *Pin, double *Pout, int colour, int check_done)
{
    const Dev &d = c->d;
    const int blocks = line_blocks((c->NJ - 1) / 2, d.sP.NW);
    bool ok = dispatch_line(d.sP, [&](auto m, auto nw) {
        launch_pdl(k_pois64<decltype(m)::value, decltype(nw)::value>, dim3(blocks), dim3(128), c->stream, d, Pin,
                   Pout, colour, check_done);
    });
    if (!ok) {
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

// One residual interval of the FP64 iteration: res_every sweeps alternating
// P -> P2 -> P, then the residual (which ends the device-side loop when done).
static int poisson64_body(fvm_ctx *c, cudaGraphConditionalHandle cond, int has_cond)
{
    Dev &d = c->d;
    for (int it = 0; it < d.res_every; it++) {
        const double *in = (it & 1) ? d.P2 : d.P;
        double *out = (it & 1) ? d.P : d.P2;
        RC(launch_pois64(c, in, out, 0, 1));
        RC(launch_pois64(c, in, out, 1, 1));
    }
    if (has_cond) launch_pdl(k_pres64<1>, dim3(c->nblk_res), dim3(256), c->stream, d, cond);
    else launch_pdl(k_pres64<0>, dim3(c->nblk_res), dim3(256), c->stream, d, cond);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

// The whole Poisson iteration as one graph.  Device loop (default): a
// while-conditional node whose body holds `groups` residual intervals; the residual
// kernel clears the condition on convergence or at the sweep cap, so the loop ends
// on the device without host synchronisation.  Host loop: the same body as a plain
// graph, replayed by the host until the control block reports completion.
static int body_groups(fvm_ctx *c, cudaGraphConditionalHandle h, int has_cond, int groups)
{
    const bool mixed = c->p.precision == FVM_MIXED;
    for (int g = 0; g < groups; g++) RC(mixed ? mixed_poisson_body(c, h, has_cond) : poisson64_body(c, h, has_cond));
    return FVM_OK;
}

static int poisson_graph(fvm_ctx *c)
{
    if (c->pgraph) return FVM_OK;
    const bool mixed = c->p.precision == FVM_MIXED;
    const int per = mixed ? c->d.refine_sweeps : c->d.res_every;
    int groups = c->p.poisson_groups > 0 ? c->p.poisson_groups : (32 + per - 1) / per;
    cudaGraph_t g = nullptr;
    cudaError_t e;
    c->pgraph_kernels = 0;
    if (c->p.poisson_host_loop) {
        FVM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        c->capturing = true;
        int rc = body_groups(c, 0, 0, groups);
        c->capturing = false;
        e = cudaStreamEndCapture(c->stream, &g);
        if (rc || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (!rc) c->err = std::string("Poisson graph capture: ") + cudaGetErrorString(e);
            return rc ? rc : FVM_ERR_CUDA;
        }
    } else {
        FVM_CUDA(c, cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle h;
        e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            c->err = std::string("Poisson loop node: ") + cudaGetErrorString(e);
            return FVM_ERR_CUDA;
        }
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            c->err = std::string("Poisson body capture: ") + cudaGetErrorString(e);
            return FVM_ERR_CUDA;
        }
        c->capturing = true;
        int rc = body_groups(c, h, 1, groups);
        c->capturing = false;
        cudaGraph_t body_out = body;
        e = cudaStreamEndCapture(c->stream, &body_out);
        if (rc || e != cudaSuccess) {
            cudaGraphDestroy(g);
            if (!rc) c->err = std::string("Poisson body capture: ") + cudaGetErrorString(e);
            return rc ? rc : FVM_ERR_CUDA;
        }
    }
    e = cudaGraphInstantiate(&c->pgraph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->err = std::string("Poisson graph instantiate: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    c->pgraph_batch = groups * per;
    return FVM_OK;
}

// Kernel launches of a finished Poisson loop (for the launch counter): whole
// bodies are launched, their kernels returning early once converged.
static long long poisson_loop_kernels(fvm_ctx *c, int niter)
{
    const int per = c->pgraph_batch;
    const bool mixed = c->p.precision == FVM_MIXED;
    long long bodies = (niter + (mixed ? 1 : 0) + per - 1) / per;
    if (bodies < 1) bodies = 1;
    return bodies * c->pgraph_kernels;
}

// Poisson phase of a step; with the device loop there is no host synchronisation
// and the statistics stay on the device (CALCCOEF copies them with the
// coefficients).
static int iter_p_async(fvm_ctx *c)
{
    Dev &d = c->d;
    k_contra_vel<<<interior_grid(c), 128, 0, c->stream>>>(d, 1);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    RC(poisson_graph(c));
    if (!c->p.poisson_host_loop) {
        FVM_CUDA(c, cudaGraphLaunch(c->pgraph, c->stream));
    } else {
        const long max_launches = (long)d.nswpp / c->pgraph_batch + 2;
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
    }
    k_bcp_ghosts<<<(c->NI + c->NJ + 127) / 128, 128, 0, c->stream>>>(d);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

// Sweep kernels alone, for timing: `sweeps` zebra sweeps that touch only scratch
// (FP64: P -> P2 both colours; MIXED: the FP32 correction without applying it),
// replayed in a graph bracketed by CUDA events on the context's stream.
static int time_sweeps(fvm_ctx *c, int sweeps, double *ms_per_launch, long long *launches)
{
    Dev &d = c->d;
    const bool mixed = c->p.precision == FVM_MIXED;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    FVM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    int rc = FVM_OK;
    for (int s = 0; s < sweeps && rc == FVM_OK; s++) {
        if (mixed) rc = mixed_sweep_pair(c, 0);
        else {
            rc = launch_pois64(c, d.P, d.P2, 0, 0);
            if (rc == FVM_OK) rc = launch_pois64(c, d.P, d.P2, 1, 0);
        }
    }
    c->capturing = false;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (!rc) c->err = std::string("sweep timing capture: ") + cudaGetErrorString(e);
        return rc ? rc : FVM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->err = std::string("sweep timing instantiate: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    FVM_CUDA(c, cudaGraphLaunch(ge, c->stream));   // warm
    FVM_CUDA(c, cudaEventRecord(c->ev_a, c->stream));
    FVM_CUDA(c, cudaGraphLaunch(ge, c->stream));
    FVM_CUDA(c, cudaEventRecord(c->ev_b, c->stream));
    FVM_CUDA(c, cudaEventSynchronize(c->ev_b));
    float ms = 0.f;
    FVM_CUDA(c, cudaEventElapsedTime(&ms, c->ev_a, c->ev_b));
    cudaGraphExecDestroy(ge);
    *launches = 2LL * sweeps;
    *ms_per_launch = ms / (2.0 * sweeps);
    c->tm.sweep_span_ms += ms;
    c->tm.sweep_span_launches += 2LL * sweeps;
    return FVM_OK;
}

int run_time_sweeps(fvm_ctx *c, int sweeps, double *ms_per_launch, long long *launches)
{
    return time_sweeps(c, sweeps, ms_per_launch, launches);
}

int run_iter_p(fvm_ctx *c, double *resid, int *sweeps)
{
    RC(iter_p_async(c));
    FVM_CUDA(c, cudaMemcpyAsync(c->h_pctl, c->d.pctl, sizeof(PCtl), cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    c->tm.kernel_launches += poisson_loop_kernels(c, c->h_pctl->niter);
    c->tm.sweeps += c->h_pctl->niter;
    int status = c->h_pctl->capped ? FVM_ERR_NOCONV : FVM_OK;
    if (!std::isfinite(c->h_pctl->resip)) {
        c->err = "non-finite Poisson residual";
        status = FVM_ERR_NAN;
    }
    if (resid) *resid = c->h_pctl->resip;
    if (sweeps) *sweeps = c->h_pctl->niter;
    return status;
}

int run_correct(fvm_ctx *c)
{
    k_grad<<<interior_grid(c), 128, 0, c->stream>>>(c->d, +1.0, 1);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_iter_t(fvm_ctx *c)
{
    k_af_su1<<<interior_grid(c), 128, 0, c->stream>>>(c->d, FVM_FIELD_T);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return predictor_sweeps(c, FVM_FIELD_T);
}

int run_calccoef(fvm_ctx *c, fvm_coeffs *out)
{
    Dev &d = c->d;
    k_calc_rows<<<(c->NJ + 127) / 128, 128, 0, c->stream>>>(d);
    KCOUNT(c);
    k_cfl<<<interior_grid(c), 128, 0, c->stream>>>(d);
    KCOUNT(c);
    fvm_coeffs *dout = reinterpret_cast<fvm_coeffs *>(d.scal + 4);
    static_assert(sizeof(fvm_coeffs) <= 12 * sizeof(double), "coeff scratch");
    k_calc_final<<<1, 1, 0, c->stream>>>(d, c->rtime, dout);
    KCOUNT(c);
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
        KCOUNT(c);
        k_explicit<<<interior_grid(c), 128, 0, c->stream>>>(d, c->p.thermal);
        KCOUNT(c);
        FVM_LAUNCH_CHECK(c);
        RC(predictor_sweeps(c, FVM_FIELD_U));
        RC(predictor_sweeps(c, FVM_FIELD_V));
        RC(run_remove_grad(c));
        RC(iter_p_async(c));
        RC(run_correct(c));
        if (c->p.thermal) RC(predictor_sweeps(c, FVM_FIELD_T));
        fvm_coeffs co;
        RC(run_calccoef(c, &co));
        c->tm.kernel_launches += poisson_loop_kernels(c, co.sweeps);
        c->tm.sweeps += co.sweeps;
        if (!std::isfinite(co.resid)) {
            c->err = "non-finite Poisson residual";
            return FVM_ERR_NAN;
        }
        if (co.resid > c->p.resimax) status = FVM_ERR_NOCONV;
        c->hist.push_back(co);
        c->tm.steps++;
        if (out) *out = co;
    }
    return status;
}

}  // namespace fvm
