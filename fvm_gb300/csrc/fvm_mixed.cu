// fvm_mixed.cu -- mixed-precision line solves: FP32 zebra sweeps and FP32 line
// solves inside FP64 defect correction.
//
// Pressure Poisson (MIXED): each outer iteration forms in FP64 the full residual
// r = SU - A P with SU = div/dt - DD(P) (iter_p.f90:24-30, 42-44) and its scaled
// L1 norm (iter_p.f90:37-50); if not converged, refine_sweeps zebra line sweeps
// solve A5 dP = r in FP32 from dP = 0 with the FP32 copies of the line factors,
// and P += dP in FP64 with the BCP ghosts (bcp.f90:19-42) refreshed from the new P.
// FP64 work per cell is one residual per refine_sweeps sweeps instead of a full
// FP64 sweep each time; the fixed point is the FP64 solution.
//
// Predictor lines (MIXED): the FP64 right-hand side C of a line (iter_u.f90:57-60)
// is solved by adi_refine passes of  r = C - T x (FP64),  T dx = r (FP32),
// x += dx (FP64), starting from the line's current values.
#include <type_traits>

#include "fvm_internal.cuh"
#include "fvm_ops.cuh"

namespace fvm {

// FP64 residual of the current P, scaled-L1 norm, FP32 right-hand side of the
// correction sweeps and zeroed correction.  The last block decides convergence.
__global__ void __launch_bounds__(256) k_mres(Dev d)
{
    __shared__ double sh[64];
    __shared__ bool last;
    if (d.pctl->done) return;
    const int it = d.pctl->niter;
    const int ni1 = d.NI - 1, total = ni1 * (d.NJ - 1);
    double ra = 0.0, pa = 0.0;
    for (int q = 0; q < 4; q++) {
        int e = blockIdx.x * 1024 + q * 256 + threadIdx.x;
        if (e < total) {
            int i = e % ni1 + 1, j = e / ni1 + 1, c = IDX(i, j);
            double su = d.DIVDT[c] - dd_p(d, d.P, i, j);
            double r = pres_at(d, d.P, su, i, j);
            ra += fabs(r);
            pa += fabs(d.cP.AP[c] * d.P[c]);
            d.RF[c] = (float)r;
            d.DF[c] = 0.0f;
        }
    }
    if (!grid_sum2(d, ra, pa, sh, last)) return;
    if (threadIdx.x == 0) {
        double resip = ra / pa;
        d.pctl->resip = resip;
        if (it > 0 && !(resip > d.resimax && it < d.nswpp)) {
            d.pctl->done = 1;
            d.pctl->capped = (resip > d.resimax) ? 1 : 0;
        } else {
            d.pctl->niter = it + d.refine_sweeps;
        }
    }
}

// One zebra colour of the FP32 correction sweep on radial rows.  With apply != 0
// (the last colour-1 sweep of an outer iteration) the warp of even row j also adds
// the correction of rows j and j-1 to P in FP64 and refreshes their BCP ghosts.
template <int M>
__global__ void __launch_bounds__(128) k_pois32(Dev d, int colour, int apply)
{
    if (d.pctl->done) return;
    const int lane = threadIdx.x & (WARP - 1);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) / WARP;
    if (w >= (d.NJ - 1) / 2) return;
    const int j = 2 * w + 1 + colour;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const LineSys &s = d.sP;
    const Coef &cf = d.cP;
    const int n = s.n;
    float v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        v[k] = 0.0f;
        if (e < n) {
            int i = e + 1, c = IDX(i, j);
            v[k] = (cf.ANf[c] * d.DF[IDX(i, jn)] + cf.ASf[c] * d.DF[IDX(i, js)]) + d.RF[c];
        }
    }
    const size_t base = size_t(j - 1) * WARP * M;
    line_apply<float, M>(v, s.invDf + base, s.faf + base, s.fbf + base, lane);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        if (e < n) d.DF[IDX(e + 1, j)] = v[k];
    }
    if (!apply) return;
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        if (e < n) {
            int i = e + 1;
            d.P[IDX(i, j)] += (double)v[k];
            d.P[IDX(i, j - 1)] += (double)d.DF[IDX(i, j - 1)];
        }
    }
    __syncwarp();
    refresh_row_ghosts<BCK_POISSON>(d, d.P, d.P, j, nullptr, nullptr, lane);
    refresh_row_ghosts<BCK_POISSON>(d, d.P, d.P, j - 1, nullptr, nullptr, lane);
}

namespace {

template <typename F>
int dispatch_m(fvm_ctx *c, int M, F &&f)
{
    switch (M) {
    case 1: f(std::integral_constant<int, 1>()); break;
    case 2: f(std::integral_constant<int, 2>()); break;
    case 3: f(std::integral_constant<int, 3>()); break;
    case 4: f(std::integral_constant<int, 4>()); break;
    case 5: f(std::integral_constant<int, 5>()); break;
    case 6: f(std::integral_constant<int, 6>()); break;
    case 7: f(std::integral_constant<int, 7>()); break;
    case 8: f(std::integral_constant<int, 8>()); break;
    case 9: f(std::integral_constant<int, 9>()); break;
    case 10: f(std::integral_constant<int, 10>()); break;
    case 11: f(std::integral_constant<int, 11>()); break;
    case 12: f(std::integral_constant<int, 12>()); break;
    case 13: f(std::integral_constant<int, 13>()); break;
    case 14: f(std::integral_constant<int, 14>()); break;
    case 15: f(std::integral_constant<int, 15>()); break;
    case 16: f(std::integral_constant<int, 16>()); break;
    default:
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

}  // namespace

int mixed_poisson_capture(fvm_ctx *c, int outer)
{
    Dev &d = c->d;
    const int half = (c->NJ - 1) / 2;
    const int blocks = (half * WARP + 127) / 128;
    for (int o = 0; o < outer; o++) {
        k_mres<<<c->nblk_res, 256, 0, c->stream>>>(d);
        KCOUNT(c);
        FVM_LAUNCH_CHECK(c);
        if (o == 0) FVM_CUDA(c, cudaEventRecordWithFlags(c->ev_a, c->stream, cudaEventRecordExternal));
        for (int s = 0; s < d.refine_sweeps; s++) {
            const int apply = (s == d.refine_sweeps - 1);
            int rc = dispatch_m(c, d.sP.M, [&](auto m) {
                k_pois32<decltype(m)::value><<<blocks, 128, 0, c->stream>>>(d, 0, 0);
                k_pois32<decltype(m)::value><<<blocks, 128, 0, c->stream>>>(d, 1, apply);
                KCOUNT(c);
                KCOUNT(c);
            });
            if (rc) return rc;
        }
        if (o == 0) {
            FVM_CUDA(c, cudaEventRecordWithFlags(c->ev_b, c->stream, cudaEventRecordExternal));
            c->span_launches = 2 * d.refine_sweeps;
        }
    }
    return FVM_OK;
}

// ---------------------------------------------------------------------------------
// Predictor lines by defect correction
// ---------------------------------------------------------------------------------
// Radial row j: -AW x(i-1) + AP x(i) - AE x(i+1) = C (AW(1)=0, AE(NI-1)=0 folded).
template <int M>
__global__ void __launch_bounds__(128) k_rad_dc(Dev d, LineSys s, Coef cf, const double *SU, double *phi, int colour,
                                                int refresh, const double *wallF, const double *farF)
{
    const int lane = threadIdx.x & (WARP - 1);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) / WARP;
    if (w >= (d.NJ - 1) / 2) return;
    const int j = 2 * w + 1 + colour;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const int n = s.n;
    if (refresh) {
        refresh_row_ghosts<BCK_DIRICHLET>(d, phi, phi, j, wallF, farF, lane);
        if (j + 1 <= d.NJ - 1) refresh_row_ghosts<BCK_DIRICHLET>(d, phi, phi, j + 1, wallF, farF, lane);
        __syncwarp();
    }
    double C[M], x[M], ap[M], aw[M], ae[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        C[k] = x[k] = ap[k] = aw[k] = ae[k] = 0.0;
        if (e < n) {
            int i = e + 1, c = IDX(i, j);
            C[k] = (cf.AN[c] * phi[IDX(i, jn)] + cf.AS[c] * phi[IDX(i, js)]) + SU[c];
            x[k] = phi[c];
            ap[k] = cf.AP[c];
            aw[k] = cf.AW[c];
            ae[k] = cf.AE[c];
        }
    }
    const size_t base = size_t(j - 1) * WARP * M;
    for (int pass = 0; pass < d.adi_refine; pass++) {
        double xl = shfl_up(x[M - 1], 1), xr = shfl_down(x[0], 1);
        if (lane == 0) xl = 0.0;
        if (lane == WARP - 1) xr = 0.0;
        float r[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            double xm = k > 0 ? x[k - 1] : xl, xp = k < M - 1 ? x[k + 1] : xr;
            r[k] = (float)(C[k] - ((ap[k] * x[k] - aw[k] * xm) - ae[k] * xp));
        }
        line_apply<float, M>(r, s.invDf + base, s.faf + base, s.fbf + base, lane);
#pragma unroll
        for (int k = 0; k < M; k++) x[k] += (double)r[k];
    }
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        if (e < n) phi[IDX(e + 1, j)] = x[k];
    }
}

// Circumferential column i, cyclic: -AS x(j-1) + AP x(j) - AN x(j+1) = C.
template <int M>
__global__ void __launch_bounds__(128) k_theta_dc(Dev d, LineSys s, Coef cf, const double *SU, double *phi,
                                                  int colour, int ghosts, const double *wallF, const double *farF)
{
    const int lane = threadIdx.x & (WARP - 1);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) / WARP;
    const int i = 2 * w + 1 + colour;
    if (i > d.NI - 1) return;
    const int n = s.n;
    double C[M], x[M], ap[M], as[M], an[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        C[k] = x[k] = ap[k] = as[k] = an[k] = 0.0;
        if (e < n) {
            int c = IDX(i, e + 1);
            C[k] = (cf.AE[c] * phi[IDX(i + 1, e + 1)] + cf.AW[c] * phi[IDX(i - 1, e + 1)]) + SU[c];
            x[k] = phi[c];
            ap[k] = cf.AP[c];
            as[k] = cf.AS[c];
            an[k] = cf.AN[c];
        }
    }
    const size_t base = size_t(i - 1) * WARP * M;
    const int ll = (n - 1) / M, lk = (n - 1) % M;
    for (int pass = 0; pass < d.adi_refine; pass++) {
        double xlast = 0.0;
#pragma unroll
        for (int k = 0; k < M; k++)
            if (k == lk) xlast = x[k];
        xlast = shfl_idx(xlast, ll);
        const double xfirst = shfl_idx(x[0], 0);
        double xl = shfl_up(x[M - 1], 1), xr = shfl_down(x[0], 1);
        if (lane == 0) xl = xlast;
        float r[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            int e = lane * M + k;
            double xm = k > 0 ? x[k - 1] : xl;
            double xp = (e == n - 1) ? xfirst : (k < M - 1 ? x[k + 1] : xr);
            r[k] = (e < n) ? (float)(C[k] - ((ap[k] * x[k] - as[k] * xm) - an[k] * xp)) : 0.0f;
        }
        line_apply<float, M>(r, s.invDf + base, s.faf + base, s.fbf + base, lane);
        line_cyclic_fix<float, M>(r, s.zf + base, s.cvf[i - 1], s.sinvf[i - 1], n, lane);
#pragma unroll
        for (int k = 0; k < M; k++) x[k] += (double)r[k];
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = lane * M + k;
        if (e < n) {
            phi[IDX(i, e + 1)] = x[k];
            if (ghosts) ghost_dirichlet(d, phi, i, e + 1, x[k], wallF, farF);
        }
    }
}

int mixed_predictor_radial(fvm_ctx *c, const LineSys &s, const Coef &cf, const double *SU, double *phi, int colour,
                           int refresh, const double *wallF, const double *farF)
{
    const int half = (c->NJ - 1) / 2;
    const int blocks = (half * WARP + 127) / 128;
    const Dev &d = c->d;
    return dispatch_m(c, s.M, [&](auto m) {
        k_rad_dc<decltype(m)::value><<<blocks, 128, 0, c->stream>>>(d, s, cf, SU, phi, colour, refresh, wallF, farF);
        KCOUNT(c);
    });
}

int mixed_predictor_theta(fvm_ctx *c, const LineSys &s, const Coef &cf, const double *SU, double *phi, int colour,
                          int ghosts, const double *wallF, const double *farF)
{
    const int nl = (c->NI - 1 + 1 - colour) / 2;
    const int blocks = (nl * WARP + 127) / 128;
    const Dev &d = c->d;
    return dispatch_m(c, s.M, [&](auto m) {
        k_theta_dc<decltype(m)::value><<<blocks, 128, 0, c->stream>>>(d, s, cf, SU, phi, colour, ghosts, wallF, farF);
        KCOUNT(c);
    });
}

}  // namespace fvm
