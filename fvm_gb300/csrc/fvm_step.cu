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

template <class S>
__global__ void k_begin(const __grid_constant__ S src)
{   // Main.f90:49-54 (full arrays); a batch advances the case's time here
    const Dev &d = dev_of(src);
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (d.btime && k == 0) *d.btime = *d.btime + d.dt;
    if (k >= d.n) return;
    d.U_N[k] = d.U[k];
    d.V_N[k] = d.V[k];
    d.T_N[k] = d.T[k];
}

template <class S>
__global__ void k_farfield_step(const __grid_constant__ S src)
{
    const Dev &d = dev_of(src);
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
template <class S>
__global__ void k_contra_vel(const __grid_constant__ S src, int with_poisson)
{
    const Dev &d = dev_of(src);
    INTERIOR_IJ
    const double *J = d.DJAC;
    int c = IDX(i, j), e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
    double ju1 = J[c] * u1_at(d, c), ju2 = J[c] * u2_at(d, c);
    double ue = 0.5 * (ju1 + J[e] * u1_at(d, e));
    // UW(1,j) = 0 in the reference (contra_vel.f90:125); with wall blowing, its flux
    double uw = (i == 1) ? d.WB[j] * d.BLOW[j] : 0.5 * (ju1 + J[w] * u1_at(d, w));
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
            d.pctl->xbase = d.XCNT[0];
            if (d.bctl && d.case_id == 0) {
                d.bctl->remaining = d.bctl->ncases;
                d.bctl->bodies = 0;
            }
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
template <class S>
__global__ void k_explicit(const __grid_constant__ S src, int thermal)
{
    const Dev &d = dev_of(src);
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
// BCU folding; the cross term of ITER_T is built from V when v_cross is set (the
// reference's iter_T.f90:89-95), else from the field itself.
template <class S>
__global__ void k_af_su2(const __grid_constant__ S src, int field, int v_cross)
{
    const Dev &d = dev_of(src);
    INTERIOR_IJ
    int c = IDX(i, j);
    FieldRefs f = field_refs(d, field);
    const double *xfield = (field == FVM_FIELD_T && v_cross) ? d.V : f.phi;
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
template <class S>
__global__ void k_grad(const __grid_constant__ S src, double sign, int with_psource)
{
    const Dev &d = dev_of(src);
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
template <class S>
__global__ void k_bcp_ghosts(const __grid_constant__ S src)
{
    const Dev &d = dev_of(src);
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
template <int M, int NW, int BCK, class S>
__global__ void __launch_bounds__(128) k_radial(const __grid_constant__ S src, int field, int colour, int refresh)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sm[G][TG * M + M * NW + 1];
    __shared__ double xch[G][2 * NW];
    const Dev &d = dev_of(src);
    if ((int)blockIdx.x * G >= (d.NJ - 1) / 2) return;   // beyond this case's lines (batch)
    const PredLine L = pred_line(d, field, 0);
    const LineSys &s = L.s;
    const Coef &cf = L.cf;
    const double *SU = L.SU, *wallF = L.wallF, *farF = L.farF;
    double *phi = L.phi;
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
template <int M, int NW, class S>
__global__ void __launch_bounds__(128) k_theta(const __grid_constant__ S src, int field, int colour, int ghosts)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sm[G][TG * M + M * NW + 1];
    __shared__ double xch[G][2 * NW];
    const Dev &d = dev_of(src);
    if (2 * (int)blockIdx.x * G + 1 + colour > d.NI - 1) return;   // beyond this case's lines (batch)
    const PredLine L = pred_line(d, field, 1);
    const LineSys &s = L.s;
    const Coef &cf = L.cf;
    const double *SU = L.SU, *wallF = L.wallF, *farF = L.farF;
    double *phi = L.phi;
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
template <int M, int NW, class S>
__global__ void __launch_bounds__(128) k_pois64(const __grid_constant__ S src, int parity, int colour, int check_done)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sm[G][TG * M + M * NW + 1];
    __shared__ double xch[G][2 * NW];
    const Dev &d = dev_of(src);
    if ((int)blockIdx.x * G >= (d.NJ - 1) / 2) return;   // beyond this case's lines (batch)
    const double *Pin = parity ? d.P2 : d.P;
    double *Pout = parity ? d.P : d.P2;
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
    // the loop's done flag is loaded together with the operands (a separate load
    // before them put one more L2 round trip on every launch's critical path)
    const int stop = check_done ? d.pctl->done : 0;
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
    if (stop) return;
    // BCP of this iteration: ghosts of P^(n-1), stored with P^n (colour 0 reads only
    // P^(n-1), so the ghosts of P^n may follow its loads)
    if (active && colour == 0 && t < WARP) {
        refresh_row_ghosts<BCK_POISSON>(d, Pin, Pout, j, nullptr, nullptr, t);
        if (j + 1 <= d.NJ - 1) refresh_row_ghosts<BCK_POISSON>(d, Pin, Pout, j + 1, nullptr, nullptr, t);
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
template <int HAS_COND, class S>
__global__ void __launch_bounds__(256) k_pres64(const __grid_constant__ S src, cudaGraphConditionalHandle cond)
{
    __shared__ double sh[64];
    __shared__ bool last;
    const Dev &d = dev_of(src);
    if ((int)blockIdx.x >= d.nblk_res64) return;   // beyond this case's blocks (batch)
    griddep_wait();
    batch_body_guard<HAS_COND>(d, cond);
    if (d.pctl->done) return;
    const int it = d.pctl->niter + d.res_every;
    const int ni1 = d.NI - 1, total = ni1 * (d.NJ - 1);
    double ra = 0.0, pa = 0.0;
#pragma unroll
    for (int q = 0; q < RES64_CELLS; q++) {
        int e = (blockIdx.x * RES64_CELLS + q) * 256 + threadIdx.x;
        if (e < total) {
            int i = e % ni1 + 1, j = e / ni1 + 1, c = IDX(i, j);
            double su = d.DIVDT[c] - dd_src(d, d.P2, i, j);
            double r = pres_at(d, d.P, su, i, j);
            ra += fabs(r);
            pa += fabs(d.cP.AP[c] * d.P[c]);
        }
    }
    griddep_launch();
    if (!grid_sum2(d, ra, pa, sh, last, d.nblk_res64)) return;
    if (threadIdx.x == 0) {
        double resip = ra / pa;
        d.pctl->niter = it;
        d.pctl->resip = resip;
        if (!(resip > d.resimax && it < d.nswpp)) {
            d.pctl->done = 1;
            d.pctl->capped = (resip > d.resimax) ? 1 : 0;
            poisson_finished<HAS_COND>(d, cond);
        }
    }
}

// ---------------------------------------------------------------------------------
// CALCCOEF (calccoef.f90:9-120): per-j wall contributions, CFL maximum, then a
// single-thread fixed-order sum (the reference's J order).
// ---------------------------------------------------------------------------------
template <class S>
__global__ void k_calc_rows(const __grid_constant__ S src)
{
    const Dev &d = dev_of(src);
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

template <class S>
__global__ void k_cfl(const __grid_constant__ S src)
{
    const Dev &d = dev_of(src);
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (j > d.NJ - 1) return;   // the whole block
    double l = 0.0;             // the CFL number is >= 0
    if (i <= d.NI - 1) {
        const int c = IDX(i, j);
        l = d.dt * (fabs(d.XIX[c] * d.U[c] + d.XIY[c] * d.V[c]) + fabs(d.ETX[c] * d.U[c] + d.ETY[c] * d.V[c]));
    }
    // the warp's maximum (exact, order-free) goes to one atomic
    for (int o = 16; o > 0; o >>= 1) l = fmax(l, __shfl_xor_sync(0xffffffffu, l, o));
    if ((threadIdx.x & 31) == 0) atomicMax(d.cflbits, (unsigned long long)__double_as_longlong(l));
}

template <class S>
__global__ void k_calc_final(const __grid_constant__ S src, double rtime, fvm_coeffs *out)
{
    const Dev &d = dev_of(src);
    if (d.bctl) {   // batch: the case's device time, one record per step and case
        rtime = *d.btime;
        out = d.bhist + (size_t)d.bctl->step * d.bctl->ncases + d.case_id;
    }
    // one warp: each lane sums every 32nd row, then a fixed shuffle tree
    double pd = 0.0, pl = 0.0, td = 0.0, tl = 0.0, nu = 0.0;
    for (int j = 1 + (int)threadIdx.x; j <= d.NJ - 1; j += 32) {
        const double *row = d.coefrow + 8 * j;
        pd = pd - row[0];
        pl = pl - row[1];
        td = td + row[2];
        tl = tl - row[3];
        nu = nu + row[4];
    }
    for (int o = 16; o > 0; o >>= 1) {
        pd += __shfl_down_sync(0xffffffffu, pd, o);
        pl += __shfl_down_sync(0xffffffffu, pl, o);
        td += __shfl_down_sync(0xffffffffu, td, o);
        tl += __shfl_down_sync(0xffffffffu, tl, o);
        nu += __shfl_down_sync(0xffffffffu, nu, o);
    }
    if (threadIdx.x != 0) return;
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
    // a negative residual reports that a bounded wait of the resident sweeps ran out
    out->resid = d.pctl->fault ? -1.0 : d.pctl->resip;
    *d.cflbits = 0ull;
}

// Batch bookkeeping after a step's CALCCOEF: the next step's records follow.
__global__ void k_batch_tick(BatchCtl *b)
{
    b->step = b->step + 1;
}

// ---------------------------------------------------------------------------------
// Host launchers.  Every launch goes to a target: one context (Dev by value) or a
// batch (Dev table, grid z = case).
// ---------------------------------------------------------------------------------
Tgt tgt_of(fvm_ctx *c)
{
    Tgt t;
    t.c = c;
    t.st = c->stream;
    t.one = &c->d;
    t.nz = 1;
    t.NI = c->NI;
    t.NJ = c->NJ;
    t.n = c->n;
    t.nblk_res = c->nblk_res;
    t.nblk_res64 = c->nblk_res64;
    t.nblk_mres = c->nblk_mres;
    t.tr = c->d.sP;
    t.tt = c->d.sUY;
    t.mixed = c->p.precision == FVM_MIXED;
    t.thermal = c->p.thermal;
    t.iter_t_bug = c->p.iter_t_bug;
    t.refine_sweeps = c->d.refine_sweeps;
    t.res_every = c->d.res_every;
    return t;
}

namespace {

inline dim3 interior_grid(const Tgt &t) { return dim3((t.NI - 1 + 127) / 128, t.NJ - 1, t.nz); }

#define RC(x)                 \
    do {                      \
        int rc_ = (x);        \
        if (rc_) return rc_;  \
    } while (0)

// Launch kernel template `kern` (instantiated for the target's Dev source) and
// count / check it.
#define LAUNCH_S(t, kern, grid, block, ...)                                   \
    do {                                                                      \
        with_src((t), [&](const auto &src_) {                                 \
            using S_ = std::decay_t<decltype(src_)>;                          \
            kern<S_><<<(grid), (block), 0, (t).st>>>(src_, ##__VA_ARGS__);    \
        });                                                                   \
        KCOUNT((t).c);                                                        \
        FVM_LAUNCH_CHECK((t).c);                                              \
    } while (0)

int line_error(fvm_ctx *c)
{
    c->err = "line length above 512 cells is not supported";
    return FVM_ERR_ARG;
}

int launch_radial(const Tgt &t, int field, int colour, int refresh)
{
    const int blocks = line_blocks((t.NJ - 1) / 2, t.tr.NW);
    bool ok = dispatch_line(t.tr, [&](auto m, auto nw) {
        with_src(t, [&](const auto &src) {
            using S = std::decay_t<decltype(src)>;
            k_radial<decltype(m)::value, decltype(nw)::value, BCK_DIRICHLET, S>
                <<<dim3(blocks, 1, t.nz), 128, 0, t.st>>>(src, field, colour, refresh);
        });
    });
    if (!ok) return line_error(t.c);
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

int launch_theta(const Tgt &t, int field, int colour, int ghosts)
{
    const int blocks = line_blocks((t.NI - 1 + 1 - colour) / 2, t.tt.NW);
    bool ok = dispatch_line(t.tt, [&](auto m, auto nw) {
        with_src(t, [&](const auto &src) {
            using S = std::decay_t<decltype(src)>;
            k_theta<decltype(m)::value, decltype(nw)::value, S>
                <<<dim3(blocks, 1, t.nz), 128, 0, t.st>>>(src, field, colour, ghosts);
        });
    });
    if (!ok) return line_error(t.c);
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

int launch_pois64(const Tgt &t, int parity, int colour, int check_done)
{
    const int blocks = line_blocks((t.NJ - 1) / 2, t.tr.NW);
    bool ok = dispatch_line(t.tr, [&](auto m, auto nw) {
        with_src(t, [&](const auto &src) {
            using S = std::decay_t<decltype(src)>;
            launch_pdl(k_pois64<decltype(m)::value, decltype(nw)::value, S>, dim3(blocks, 1, t.nz), dim3(128), t.st,
                       src, parity, colour, check_done);
        });
    });
    if (!ok) return line_error(t.c);
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

// One residual interval of the FP64 iteration: res_every sweeps alternating
// P -> P2 -> P, then the residual (which ends the device-side loop when done).
int poisson64_body(const Tgt &t, cudaGraphConditionalHandle cond, int has_cond)
{
    for (int it = 0; it < t.res_every; it++) {
        RC(launch_pois64(t, it & 1, 0, 1));
        RC(launch_pois64(t, it & 1, 1, 1));
    }
    with_src(t, [&](const auto &src) {
        using S = std::decay_t<decltype(src)>;
        if (has_cond) launch_pdl(k_pres64<1, S>, dim3(t.nblk_res64, 1, t.nz), dim3(256), t.st, src, cond);
        else launch_pdl(k_pres64<0, S>, dim3(t.nblk_res64, 1, t.nz), dim3(256), t.st, src, cond);
    });
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

}  // namespace

// The predictor of one field after its first-factor SU is in place.
int predictor_sweeps(const Tgt &t, int field)
{
    const bool tk = field == FVM_FIELD_T;
    // sweep 1 (radial lines), ghosts refreshed from the pre-sweep field (BCU)
    for (int colour = 0; colour < 2; colour++) {
        if (t.mixed) RC(mixed_predictor_radial(t, field, colour, colour == 0));
        else RC(launch_radial(t, field, colour, colour == 0));
    }
    // second factor right-hand side from the first-sweep field
    LAUNCH_S(t, k_af_su2, interior_grid(t), 128, field, (tk && t.iter_t_bug) ? 1 : 0);
    for (int colour = 0; colour < 2; colour++) {
        if (t.mixed) RC(mixed_predictor_theta(t, field, colour, tk ? 1 : 0));
        else RC(launch_theta(t, field, colour, tk ? 1 : 0));
    }
    return FVM_OK;
}

// Main.f90:48-93 up to the Poisson loop: step start, far-field values, fluxes,
// explicit terms, the U and V predictors, the gradient removal and the Poisson
// source.
int step_before_poisson(const Tgt &t)
{
    LAUNCH_S(t, k_begin, dim3((t.n + 255) / 256, 1, t.nz), 256);
    LAUNCH_S(t, k_farfield_step, dim3((t.NJ + 127) / 128, 1, t.nz), 128);
    LAUNCH_S(t, k_contra_vel, interior_grid(t), 128, 0);
    LAUNCH_S(t, k_explicit, interior_grid(t), 128, t.thermal);
    RC(predictor_sweeps(t, FVM_FIELD_U));
    RC(predictor_sweeps(t, FVM_FIELD_V));
    LAUNCH_S(t, k_grad, interior_grid(t), 128, -1.0, 0);
    LAUNCH_S(t, k_contra_vel, interior_grid(t), 128, 1);
    return FVM_OK;
}

// `groups` residual intervals of the Poisson iteration.
int poisson_bodies(const Tgt &t, cudaGraphConditionalHandle h, int has_cond, int groups)
{
    for (int g = 0; g < groups; g++) RC(t.mixed ? mixed_poisson_body(t, h, has_cond) : poisson64_body(t, h, has_cond));
    return FVM_OK;
}

// Main.f90:93-114 after the Poisson loop: BCP ghosts, correction, ITER_T and the
// CALCCOEF kernels (a single context's record goes to dout; a batch appends one
// record per case to its history).
int step_after_poisson(const Tgt &t, double rtime, fvm_coeffs *dout)
{
    LAUNCH_S(t, k_bcp_ghosts, dim3((t.NI + t.NJ + 127) / 128, 1, t.nz), 128);
    LAUNCH_S(t, k_grad, interior_grid(t), 128, +1.0, 1);
    if (t.thermal) RC(predictor_sweeps(t, FVM_FIELD_T));
    LAUNCH_S(t, k_calc_rows, dim3((t.NJ + 127) / 128, 1, t.nz), 128);
    LAUNCH_S(t, k_cfl, interior_grid(t), 128);
    LAUNCH_S(t, k_calc_final, dim3(1, 1, t.nz), 32, rtime, dout);
    return FVM_OK;
}

// `sweeps` zebra sweeps that touch only scratch (FP64: P -> P2 both colours;
// MIXED: the FP32 correction without applying it), for timing.
int sweep_pairs(const Tgt &t, int sweeps)
{
    if (t.mixed && !t.tab.devs && t.c->res_lines)   // all sweeps in one resident launch
        return resident_sweeps(t, sweeps, 0, 0, 0u, 0, 0, 0);
    for (int s = 0; s < sweeps; s++) {
        if (t.mixed) RC(mixed_sweep_pair(t, 0));
        else {
            RC(launch_pois64(t, 0, 0, 0));
            RC(launch_pois64(t, 0, 1, 0));
        }
    }
    return FVM_OK;
}

// `sweeps` circumferential predictor sweeps of a field (both colours), for timing.
int theta_pairs(const Tgt &t, int field, int sweeps)
{
    for (int s = 0; s < sweeps; s++)
        for (int colour = 0; colour < 2; colour++) {
            if (t.mixed) RC(mixed_predictor_theta(t, field, colour, 0));
            else RC(launch_theta(t, field, colour, 0));
        }
    return FVM_OK;
}

int launch_batch_tick(const Tgt &t, BatchCtl *b)
{
    k_batch_tick<<<1, 1, 0, t.st>>>(b);
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

int run_begin_step(fvm_ctx *c)
{
    c->rtime = c->rtime + c->p.dt;
    c->niter_time += 1;
    Tgt t = tgt_of(c);
    LAUNCH_S(t, k_begin, dim3((t.n + 255) / 256, 1, 1), 256);
    LAUNCH_S(t, k_farfield_step, dim3((t.NJ + 127) / 128, 1, 1), 128);
    return FVM_OK;
}

int run_contra_vel(fvm_ctx *c)
{
    Tgt t = tgt_of(c);
    LAUNCH_S(t, k_contra_vel, interior_grid(t), 128, 0);
    return FVM_OK;
}

int run_nl(fvm_ctx *c, int field)
{
    k_nl<<<interior_grid(tgt_of(c)), 128, 0, c->stream>>>(c->d, field);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_dif(fvm_ctx *c, int field)
{
    k_dif<<<interior_grid(tgt_of(c)), 128, 0, c->stream>>>(c->d, field);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_p_source(fvm_ctx *c)
{
    k_psource<<<interior_grid(tgt_of(c)), 128, 0, c->stream>>>(c->d);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

int run_iter_u(fvm_ctx *c, int field)
{
    k_af_su1<<<interior_grid(tgt_of(c)), 128, 0, c->stream>>>(c->d, field);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return predictor_sweeps(tgt_of(c), field);
}

int run_remove_grad(fvm_ctx *c)
{
    Tgt t = tgt_of(c);
    LAUNCH_S(t, k_grad, interior_grid(t), 128, -1.0, 0);
    return FVM_OK;
}

namespace {

// The whole Poisson iteration of a context as one graph.  Device loop: a
// while-conditional node whose body holds `groups` residual intervals; the residual
// kernel clears the condition on convergence or at the sweep cap, so the loop ends
// on the device without host synchronisation.  Host loop (default): the same body
// as a plain graph, replayed by the host until the control block reports
// completion (profilers can then see each kernel).
int poisson_graph_build(fvm_ctx *c);

// The resident sweep launch carries the cooperative attribute (all blocks
// co-resident); if the graph cannot hold it, the graph is built again without the
// attribute (the blocks then fit by the occupancy check of resident_setup, and
// every wait is bounded either way).
int poisson_graph(fvm_ctx *c)
{
    if (c->pgraph) return FVM_OK;
    int rc = poisson_graph_build(c);
    if (rc == FVM_ERR_CUDA && c->res_lines && c->res_coop) {
        cudaGetLastError();
        c->res_coop = false;
        rc = poisson_graph_build(c);
    }
    return rc;
}

int poisson_graph_build(fvm_ctx *c)
{
    Tgt t = tgt_of(c);
    const int per = t.mixed ? t.refine_sweeps : t.res_every;
    int groups = c->p.poisson_groups > 0 ? c->p.poisson_groups : (32 + per - 1) / per;
    cudaGraph_t g = nullptr;
    cudaError_t e;
    c->pgraph_kernels = 0;
    if (c->p.poisson_host_loop) {
        FVM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        c->capturing = true;
        int rc = poisson_bodies(t, 0, 0, groups);
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
        int rc = poisson_bodies(t, h, 1, groups);
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
long long poisson_loop_kernels(fvm_ctx *c, int niter)
{
    const int per = c->pgraph_batch;
    const bool mixed = c->p.precision == FVM_MIXED;
    long long bodies = (niter + (mixed ? 1 : 0) + per - 1) / per;
    if (bodies < 1) bodies = 1;
    return bodies * c->pgraph_kernels;
}

// The Poisson loop of a context after its source term is in place; with the
// device loop there is no host synchronisation and the statistics stay on the
// device (CALCCOEF copies them with the coefficients).
int poisson_loop(fvm_ctx *c)
{
    Dev &d = c->d;
    RC(poisson_graph(c));
    if (!c->p.poisson_host_loop) {
        FVM_CUDA(c, cudaGraphLaunch(c->pgraph, c->stream));
        return FVM_OK;
    }
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
    return FVM_OK;
}

// Sweep kernels alone, for timing: `sweeps` zebra sweeps that touch only scratch,
// replayed in a graph bracketed by CUDA events on the context's stream.
int time_sweeps(fvm_ctx *c, int sweeps, double *ms_per_launch, long long *launches)
{
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    FVM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->capturing = true;
    int rc = sweep_pairs(tgt_of(c), sweeps);
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
    const bool resident = c->p.precision == FVM_MIXED && c->res_lines;
    *launches = resident ? 1LL : 2LL * sweeps;
    *ms_per_launch = ms / (2.0 * sweeps);   // per zebra colour
    c->tm.sweep_span_ms += ms;
    c->tm.sweep_span_launches += *launches;
    return FVM_OK;
}

int calccoef_copy(fvm_ctx *c, fvm_coeffs *dout, fvm_coeffs *out)
{
    FVM_CUDA(c, cudaMemcpyAsync(&c->last, dout, sizeof(fvm_coeffs), cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (out) *out = c->last;
    if (!std::isfinite(c->last.cd) || !std::isfinite(c->last.cl)) {
        c->err = "non-finite drag or lift";
        return FVM_ERR_NAN;
    }
    return FVM_OK;
}

// A bounded wait of the resident sweeps ran out: clear the exchange state so the
// context stays usable, and report it.
int resident_fault(fvm_ctx *c)
{
    RC(resident_reset(c));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    c->err = "resident Poisson sweeps: a bounded wait for a neighbouring block ran out";
    return FVM_ERR_TIMEOUT;
}

fvm_coeffs *coef_slot(fvm_ctx *c)
{
    static_assert(sizeof(fvm_coeffs) <= 12 * sizeof(double), "coeff scratch");
    return reinterpret_cast<fvm_coeffs *>(c->d.scal + 4);
}

}  // namespace

int run_time_sweeps(fvm_ctx *c, int sweeps, double *ms_per_launch, long long *launches)
{
    return time_sweeps(c, sweeps, ms_per_launch, launches);
}

// Two resident sweeps on scratch with exchange tags no block publishes: every
// wait at the second sweep runs out after max_polls polls.
int run_resident_wait_test(fvm_ctx *c, int max_polls)
{
    if (c->p.precision != FVM_MIXED || !c->res_lines) {
        c->err = "the context does not use the resident sweep path";
        return FVM_ERR_ARG;
    }
    // four sweeps: waits at sweeps 2-4 (one exchange per sweep) or at sweep 3 (per pair)
    RC(resident_sweeps(tgt_of(c), 4, 0, max_polls, 0x40000000u, 0, 0, 0));
    FVM_CUDA(c, cudaMemcpyAsync(c->h_pctl, c->d.pctl, sizeof(PCtl), cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!c->h_pctl->fault) {
        c->err = "a wait that cannot be satisfied did not report";
        return FVM_ERR_CUDA;
    }
    return resident_fault(c);
}

int run_iter_p(fvm_ctx *c, double *resid, int *sweeps)
{
    Tgt t = tgt_of(c);
    LAUNCH_S(t, k_contra_vel, interior_grid(t), 128, 1);
    RC(poisson_loop(c));
    LAUNCH_S(t, k_bcp_ghosts, dim3((t.NI + t.NJ + 127) / 128, 1, 1), 128);
    FVM_CUDA(c, cudaMemcpyAsync(c->h_pctl, c->d.pctl, sizeof(PCtl), cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    c->tm.kernel_launches += poisson_loop_kernels(c, c->h_pctl->niter);
    c->tm.sweeps += c->h_pctl->niter;
    if (c->h_pctl->fault) return resident_fault(c);
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
    Tgt t = tgt_of(c);
    LAUNCH_S(t, k_grad, interior_grid(t), 128, +1.0, 1);
    return FVM_OK;
}

int run_iter_t(fvm_ctx *c)
{
    k_af_su1<<<interior_grid(tgt_of(c)), 128, 0, c->stream>>>(c->d, FVM_FIELD_T);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return predictor_sweeps(tgt_of(c), FVM_FIELD_T);
}

int run_calccoef(fvm_ctx *c, fvm_coeffs *out)
{
    Tgt t = tgt_of(c);
    fvm_coeffs *dout = coef_slot(c);
    LAUNCH_S(t, k_calc_rows, dim3((t.NJ + 127) / 128, 1, 1), 128);
    LAUNCH_S(t, k_cfl, interior_grid(t), 128);
    LAUNCH_S(t, k_calc_final, dim3(1, 1, 1), 32, c->rtime, dout);
    const double cl_prev = c->last.cl;   // CL_NM1 (calccoef.f90:109)
    fvm_coeffs co;
    RC(calccoef_copy(c, dout, &co));
    if (out) *out = co;
    return post_after_calccoef(c, cl_prev, co);
}

int run_step(fvm_ctx *c, int nsteps, fvm_coeffs *out)
{
    int status = FVM_OK;
    c->hist.clear();
    Tgt t = tgt_of(c);
    for (int s = 0; s < nsteps; s++) {
        c->rtime = c->rtime + c->p.dt;
        c->niter_time += 1;
        RC(step_before_poisson(t));
        RC(poisson_loop(c));
        fvm_coeffs *dout = coef_slot(c);
        RC(step_after_poisson(t, c->rtime, dout));
        const double cl_prev = c->last.cl;   // CL_NM1 (calccoef.f90:109)
        fvm_coeffs co;
        RC(calccoef_copy(c, dout, &co));
        if (co.resid < 0.0) return resident_fault(c);
        RC(post_after_calccoef(c, cl_prev, co));
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
