// fvm_mixed.cu -- mixed-precision line solves: FP32 zebra sweeps and FP32 line
// solves inside FP64 defect correction.
//
// Pressure Poisson (MIXED): each outer iteration forms the full residual
// r = SU - A P with SU = div/dt - DD(P) (iter_p.f90:24-30, 42-44) of the FP64 P in
// double-float (FP32 pairs, ~2^-46 relative per term) and its scaled L1 norm
// (iter_p.f90:37-50); if not converged, refine_sweeps zebra line sweeps solve
// A5 dP = r in FP32 from dP = 0 with the FP32 copies of the line factors, and
// P += dP in FP64 with the BCP ghosts (bcp.f90:19-42) refreshed from the new P.
// The fixed point is the FP64 solution to the residual's double-float rounding,
// far below any Poisson tolerance; no FP64 sweep runs.
//
// Predictor lines (MIXED): the FP64 right-hand side C of a line (iter_u.f90:57-60)
// is solved by adi_refine passes of  r = C - T x (FP64),  T dx = r (FP32),
// x += dx (FP64), starting from the line's current values.
#include <type_traits>

#include "fvm_internal.cuh"
#include "fvm_ops.cuh"
#include "fvm_df.cuh"

namespace fvm {

// The pressure-equation coefficients and cross-term weights split into
// double-float planes for k_mres (dd_split: hi + lo within 2^-46 of the FP64 value).
__global__ void k_pcoef_df(Dev d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const double *src[9] = {d.cP.AE, d.cP.AW, d.cP.AN, d.cP.AS, d.cP.AP, d.CNE, d.CSE, d.CNW, d.CSW};
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const dd v = dd_split(src[k][c]);
        d.PCD[size_t(k) * d.n + c] = make_float2(v.hi, v.lo);
    }
}

void split_pcoef(fvm_ctx *c)
{
    k_pcoef_df<<<(c->n + 255) / 256, 256, 0, c->stream>>>(c->d);
}

// Residual of the current P (iter_p.f90:24-30, 42-44: SU = DIVDT - DD(P), then the
// five-point residual), its scaled-L1 norm (iter_p.f90:37-50), the FP32 right-hand
// side of the correction sweeps and the zeroed correction.  The last block decides
// convergence.
//
// Evaluated in double-float (the terms and order of dd_src and pres_at): about
// 2^-46 relative to |AP P| per term, far below any Poisson tolerance, on the FP32
// pipes instead of GB300's narrow FP64 pipe.  A block owns a tile of MRES_TI x
// MRES_TJ cells; the pressure of the tile and of its halo (two cells below, one
// above, in both directions: the positional cross term reaches (i-2, j-2)) is split
// once into shared memory, the coefficients come pre-split (d.PCD), and the two
// norms are summed in FP32 up to the warp and in FP64 beyond.  DECIDE = 0 (the
// single-context resident path) leaves the block sums in d.partial for the resident
// sweep launch to decide convergence (resident_decide); DECIDE = 1 decides here.
template <int HAS_COND, class S, int DECIDE>
__global__ void __launch_bounds__(256, 6) k_mres(const __grid_constant__ S src, cudaGraphConditionalHandle cond)
{
    constexpr int TI = MRES_TI, TJ = MRES_TJ, W = TI + 3, H = TJ + 3;
    static_assert(TI == WARP && TI * TJ == 256, "one warp per tile row");
    __shared__ double sh[64];
    __shared__ bool last;
    __shared__ float2 ps[H][W];
    const Dev &d = dev_of(src);
    if ((int)blockIdx.x >= d.nblk_mres) return;   // beyond this case's blocks (batch)
    const int ti = (d.NI - 1 + TI - 1) / TI;
    const int i0 = (blockIdx.x % ti) * TI + 1, j0 = (blockIdx.x / ti) * TJ + 1;   // first cell of the tile
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = i0 + tx, j = j0 + ty;
    const bool inside = i <= d.NI - 1 && j <= d.NJ - 1;
    // dd_src: the weights of (i,j), or of (i-1,j-1) (zero on row/column 1)
    const bool has_cross = inside && (!d.dd_pos || (i > 1 && j > 1));
    const int c = inside ? IDX(i, j) : 0;
    const int cc = d.dd_pos ? (has_cross ? IDX(i - 1, j - 1) : 0) : c;
    // the coefficient planes are written at set-up only: loaded before the wait for
    // the preceding kernel
    float2 cf[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const bool ok = k < 5 ? inside : has_cross;
        cf[k] = ok ? d.PCD[size_t(k) * d.n + (k < 5 ? c : cc)] : make_float2(0.0f, 0.0f);
    }
    griddep_wait();
    batch_body_guard<HAS_COND>(d, cond);
    if (d.pctl->done) return;
    const int it = d.pctl->niter;
    const double *P = d.P;
    const double divdt = inside ? d.DIVDT[c] : 0.0;
    for (int k = threadIdx.x; k < H * W; k += 256) {   // rows j0-2 .. j0+TJ, columns i0-2 .. i0+TI
        const int r = k / W, q = k - r * W;
        const int ih = i0 - 2 + q, jh = j0 - 2 + r;
        dd v(0.0f, 0.0f);
        if (ih >= 0 && ih <= d.NI && jh >= 0 && jh <= d.NJ) v = dd_split(P[IDX(ih, jh)]);
        ps[r][q] = make_float2(v.hi, v.lo);
    }
    __syncthreads();
    float raf = 0.0f, paf = 0.0f;
    if (inside) {
        auto at = [&](int a, int b) {   // P(i + a, j + b), rows as stored (ghost rows included)
            const float2 v = ps[ty + 2 + b][tx + 2 + a];
            return dd(v.x, v.y);
        };
        auto co = [&](int k) { return dd(cf[k].x, cf[k].y); };
        dd cross = dd(0.0f, 0.0f);
        if (!d.dd_pos) {
            cross = ((co(5) * at(1, 1) + co(6) * at(1, -1)) + co(7) * at(-1, 1)) + co(8) * at(-1, -1);
        } else if (has_cross) {
            cross = ((co(5) * at(0, 0) + co(6) * at(0, -2)) + co(7) * at(-2, 0)) + co(8) * at(-2, -2);
        }
        // circumferential neighbours through the periodic wrap (jwrap), as pres_at
        const dd pn = (j + 1 == d.NJ) ? dd_split(P[IDX(i, 1)]) : at(0, 1);
        const dd pso = (j == 1) ? dd_split(P[IDX(i, d.NJ - 1)]) : at(0, -1);
        const dd su = dd_split(divdt) - cross;
        const dd app = co(4) * at(0, 0);
        const dd r = ((((co(0) * at(1, 0) + co(1) * at(-1, 0)) + co(2) * pn) + co(3) * pso) + su) - app;
        raf = fabsf(r.hi);
        paf = fabsf(app.hi);
        d.RF[c] = r.hi;
        d.DF[c] = 0.0f;
    }
    griddep_launch();
    double ra, pa;
    if (!DECIDE) {
        block_sum2f(raf, paf, ra, pa, sh);
        if (threadIdx.x == 0) {
            d.partial[2 * blockIdx.x] = ra;
            d.partial[2 * blockIdx.x + 1] = pa;
        }
        return;
    }
    if (!grid_sum2f(d, raf, paf, ra, pa, sh, last, d.nblk_mres)) return;
    if (threadIdx.x == 0) {
        double resip = ra / pa;
        d.pctl->resip = resip;
        if (it > 0 && !(resip > d.resimax && it < d.nswpp)) {
            d.pctl->done = 1;
            d.pctl->capped = (resip > d.resimax) ? 1 : 0;
            poisson_finished<HAS_COND>(d, cond);
        } else {
            d.pctl->niter = it + d.refine_sweeps;
        }
    }
}

// One zebra colour of the FP32 correction sweep on radial rows.  With apply != 0
// (the last colour-1 sweep of an outer iteration) the warp of even row j also adds
// the correction of rows j and j-1 to P in FP64 and refreshes their BCP ghosts.
template <int M, int NW, class S>
__global__ void __launch_bounds__(128) k_pois32(const __grid_constant__ S src, int colour, int apply, int check_done)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ float sm[G][TG * M + M * NW + 1];
    __shared__ float xch[G][2 * NW];
    const Dev &d = dev_of(src);
    if ((int)blockIdx.x * G >= (d.NJ - 1) / 2) return;   // beyond this case's lines (batch)
    int gl, t, gib;
    group_of<NW>(gl, t, gib);
    const bool active = gl < (d.NJ - 1) / 2;
    const int j = active ? 2 * gl + 1 + colour : 1;
    const int jn = jwrap(d, j + 1), js = jwrap(d, j - 1);
    const LineSys &s = d.sP;
    const Coef &cf = d.cP;
    const int n = s.n;
    // constants first: line factors and coupling coefficients
    const size_t base = size_t(j - 1) * TG * M;
    float fi[M], fa[M], fb[M], an[M], as[M];
    load_factors<float, M, NW>(fi, fa, fb, s.invDf + base, s.faf + base, s.fbf + base, t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        bool ok = active && e < n;
        an[k] = ok ? cf.ANf[IDX(e + 1, j)] : 0.0f;
        as[k] = ok ? cf.ASf[IDX(e + 1, j)] : 0.0f;
    }
    griddep_wait();
    // the loop's done flag is loaded together with the operands (a separate load
    // before them put one more L2 round trip on every launch's critical path)
    const int stop = check_done ? d.pctl->done : 0;
    float v[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        v[k] = 0.0f;
        if (active && e < n) {
            int i = e + 1;
            v[k] = pois32_rhs(an[k], d.DF[IDX(i, jn)], as[k], d.DF[IDX(i, js)], d.RF[IDX(i, j)]);
        }
    }
    if (stop) return;
    griddep_launch();   // the next sweep may start its constant prologue now
    to_chunks<float, M, NW>(v, sm[gib], t);
    group_apply_r<float, M, NW>(v, fi, fa, fb, t, xch[gib]);
    to_interleaved<float, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) d.DF[IDX(e + 1, j)] = v[k];
    }
    if (!apply) return;
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) {
            int i = e + 1;
            d.P[IDX(i, j)] += (double)v[k];
            d.P[IDX(i, j - 1)] += (double)d.DF[IDX(i, j - 1)];
        }
    }
    gsync<NW>();
    if (active && t < WARP) {
        refresh_row_ghosts<BCK_POISSON>(d, d.P, d.P, j, nullptr, nullptr, t);
        refresh_row_ghosts<BCK_POISSON>(d, d.P, d.P, j - 1, nullptr, nullptr, t);
    }
}

// One zebra sweep of the FP32 correction (both colours); apply != 0 also adds the
// correction to P.  check_done is off when the pair is replayed for timing.
static int sweep_pair(const Tgt &t, int apply, int check_done)
{
    const int blocks = line_blocks((t.NJ - 1) / 2, t.tr.NW);
    bool ok = dispatch_line(t.tr, [&](auto m, auto nw) {
        with_src(t, [&](const auto &src) {
            using S = std::decay_t<decltype(src)>;
            auto k = k_pois32<decltype(m)::value, decltype(nw)::value, S>;
            launch_pdl(k, dim3(blocks, 1, t.nz), dim3(128), t.st, src, 0, 0, check_done);
            launch_pdl(k, dim3(blocks, 1, t.nz), dim3(128), t.st, src, 1, apply, check_done);
        });
    });
    if (!ok) {
        t.c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    KCOUNT(t.c);
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

int mixed_sweep_pair(const Tgt &t, int apply) { return sweep_pair(t, apply, 0); }

// One FP32 correction sweep of the per-colour path on the current state, whatever
// path the context's step uses (tests compare the two paths).
int mixed_sweep_percolour(const Tgt &t, int apply) { return sweep_pair(t, apply, 0); }

// One outer iteration of the MIXED Poisson: residual (ends the device-side
// loop when converged or capped), then refine_sweeps FP32 zebra sweeps, the last
// of which adds the correction to P.
int mixed_poisson_body(const Tgt &t, cudaGraphConditionalHandle cond, int has_cond)
{
    // one context with resident sweeps: the interval in one resident launch, which
    // also takes the convergence decision from the residual's block sums
    const bool resident = !t.tab.devs && t.c->res_lines;
    with_src(t, [&](const auto &src) {
        using S = std::decay_t<decltype(src)>;
        const dim3 g(t.nblk_mres, 1, t.nz);
        if (resident) launch_pdl(k_mres<0, S, 0>, g, dim3(256), t.st, src, cond);
        else if (has_cond) launch_pdl(k_mres<1, S, 1>, g, dim3(256), t.st, src, cond);
        else launch_pdl(k_mres<0, S, 1>, g, dim3(256), t.st, src, cond);
    });
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    if (resident) return resident_sweeps(t, t.refine_sweeps, 1, 0, 0u, cond, has_cond, 1, 1);
    for (int s = 0; s < t.refine_sweeps; s++) {
        int rc = sweep_pair(t, s == t.refine_sweeps - 1, 1);
        if (rc) return rc;
    }
    return FVM_OK;
}

// ---------------------------------------------------------------------------------
// Predictor lines by defect correction
// ---------------------------------------------------------------------------------
// Radial row j: -AW x(i-1) + AP x(i) - AE x(i+1) = C (AW(1)=0, AE(NI-1)=0 folded).
// The line's FP64 values are staged in shared memory in natural order so that the
// defect r = C - T x reads its neighbours there.
template <int M, int NW, class S>
__global__ void __launch_bounds__(128) k_rad_dc(const __grid_constant__ S src, int field, int colour, int refresh)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sx[G][TG * M + M * NW + 1];
    __shared__ float sm[G][TG * M + M * NW + 1];
    __shared__ float xch[G][2 * NW];
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
        refresh_row_ghosts<BCK_DIRICHLET>(d, phi, phi, j, wallF, farF, t);
        if (j + 1 <= d.NJ - 1) refresh_row_ghosts<BCK_DIRICHLET>(d, phi, phi, j + 1, wallF, farF, t);
    }
    double C[M], x[M], ap[M], aw[M], ae[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        C[k] = x[k] = ap[k] = aw[k] = ae[k] = 0.0;
        if (active && e < n) {
            int i = e + 1, c = IDX(i, j);
            C[k] = (cf.AN[c] * phi[IDX(i, jn)] + cf.AS[c] * phi[IDX(i, js)]) + SU[c];
            x[k] = phi[c];
            ap[k] = cf.AP[c];
            aw[k] = cf.AW[c];
            ae[k] = cf.AE[c];
        }
    }
    const size_t base = size_t(j - 1) * TG * M;
    for (int pass = 0; pass < d.adi_refine; pass++) {
#pragma unroll
        for (int k = 0; k < M; k++) sx[gib][spad(k * TG + t)] = x[k];
        gsync<NW>();
        float r[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            int e = k * TG + t;
            double xm = e > 0 ? sx[gib][spad(e - 1)] : 0.0;
            double xp = e + 1 < n ? sx[gib][spad(e + 1)] : 0.0;
            r[k] = (e < n) ? (float)(C[k] - ((ap[k] * x[k] - aw[k] * xm) - ae[k] * xp)) : 0.0f;
        }
        gsync<NW>();
        to_chunks<float, M, NW>(r, sm[gib], t);
        group_apply<float, M, NW>(r, s.invDf + base, s.faf + base, s.fbf + base, t, xch[gib]);
        to_interleaved<float, M, NW>(r, sm[gib], t);
#pragma unroll
        for (int k = 0; k < M; k++) x[k] += (double)r[k];
    }
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) phi[IDX(e + 1, j)] = x[k];
    }
}

// Circumferential column i, cyclic: -AS x(j-1) + AP x(j) - AN x(j+1) = C.
template <int M, int NW, class S>
__global__ void __launch_bounds__(128) k_theta_dc(const __grid_constant__ S src, int field, int colour, int ghosts)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ double sx[G][TG * M + M * NW + 1];
    __shared__ float sm[G][TG * M + M * NW + 1];
    __shared__ float xch[G][2 * NW];
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
    double C[M], x[M], ap[M], as[M], an[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        C[k] = x[k] = ap[k] = as[k] = an[k] = 0.0;
        if (active && e < n) {
            int c = IDX(i, e + 1);
            C[k] = (cf.AE[c] * phi[IDX(i + 1, e + 1)] + cf.AW[c] * phi[IDX(i - 1, e + 1)]) + SU[c];
            x[k] = phi[c];
            ap[k] = cf.AP[c];
            as[k] = cf.AS[c];
            an[k] = cf.AN[c];
        }
    }
    const size_t base = size_t(i - 1) * TG * M;
    for (int pass = 0; pass < d.adi_refine; pass++) {
#pragma unroll
        for (int k = 0; k < M; k++) sx[gib][spad(k * TG + t)] = x[k];
        gsync<NW>();
        float r[M];
#pragma unroll
        for (int k = 0; k < M; k++) {
            int e = k * TG + t;
            double xm = sx[gib][spad(e > 0 ? e - 1 : n - 1)];
            double xp = sx[gib][spad(e + 1 < n ? e + 1 : 0)];
            r[k] = (e < n) ? (float)(C[k] - ((ap[k] * x[k] - as[k] * xm) - an[k] * xp)) : 0.0f;
        }
        gsync<NW>();
        to_chunks<float, M, NW>(r, sm[gib], t);
        group_apply<float, M, NW>(r, s.invDf + base, s.faf + base, s.fbf + base, t, xch[gib]);
        group_cyclic_fix<float, M, NW>(r, s.zf + base, s.cvf[i - 1], s.sinvf[i - 1], n, t, xch[gib]);
        to_interleaved<float, M, NW>(r, sm[gib], t);
#pragma unroll
        for (int k = 0; k < M; k++) x[k] += (double)r[k];
    }
#pragma unroll
    for (int k = 0; k < M; k++) {
        int e = k * TG + t;
        if (active && e < n) {
            phi[IDX(i, e + 1)] = x[k];
            if (ghosts) ghost_dirichlet(d, phi, i, e + 1, x[k], wallF, farF);
        }
    }
}

int mixed_predictor_radial(const Tgt &t, int field, int colour, int refresh)
{
    const int blocks = line_blocks((t.NJ - 1) / 2, t.tr.NW);
    bool ok = dispatch_line(t.tr, [&](auto m, auto nw) {
        with_src(t, [&](const auto &src) {
            using S = std::decay_t<decltype(src)>;
            k_rad_dc<decltype(m)::value, decltype(nw)::value, S>
                <<<dim3(blocks, 1, t.nz), 128, 0, t.st>>>(src, field, colour, refresh);
        });
    });
    if (!ok) {
        t.c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

int mixed_predictor_theta(const Tgt &t, int field, int colour, int ghosts)
{
    const int blocks = line_blocks((t.NI - 1 + 1 - colour) / 2, t.tt.NW);
    bool ok = dispatch_line(t.tt, [&](auto m, auto nw) {
        with_src(t, [&](const auto &src) {
            using S = std::decay_t<decltype(src)>;
            k_theta_dc<decltype(m)::value, decltype(nw)::value, S>
                <<<dim3(blocks, 1, t.nz), 128, 0, t.st>>>(src, field, colour, ghosts);
        });
    });
    if (!ok) {
        t.c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    KCOUNT(t.c);
    FVM_LAUNCH_CHECK(t.c);
    return FVM_OK;
}

}  // namespace fvm
