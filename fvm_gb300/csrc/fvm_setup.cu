// fvm_setup.cu -- one-time setup of a context: device slab, GRID/METRIC/INIT on the
// device (FP64), the constant five-point coefficient sets of every line solve with
// their boundary folding, and the precomputed tridiagonal factors of every line.
#include <cmath>
#include <cstring>

#include "fvm_internal.cuh"

namespace fvm {

// ---------------------------------------------------------------------------------
// Slab allocation
// ---------------------------------------------------------------------------------
namespace {

struct Bump {
    char *base;
    size_t off = 0;
    template <typename T>
    T *take(size_t count)
    {
        off = (off + 255) & ~size_t(255);
        T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
};

// Line tile of a family: warps per line group and elements per thread, either
// given (both > 0, validated when the context is created) or derived from n.
void carve_sys(Bump &b, LineSys &s, int lines, int n, int cyclic, int nw, int m)
{
    s.lines = lines;
    s.n = n;
    s.NW = nw > 0 ? nw : group_warps(n);
    s.M = m > 0 ? m : (n + WARP * s.NW - 1) / (WARP * s.NW);
    s.cyclic = cyclic;
    // capacity for the largest tile (4 warps x 4 elements), so that the tile can
    // be changed later without reallocation; the layout in use is dense
    size_t cnt = size_t(lines) * WARP * 4 * 4;
    s.invD = b.take<double>(cnt);
    s.fa = b.take<double>(cnt);
    s.fb = b.take<double>(cnt);
    s.invDf = b.take<float>(cnt);
    s.faf = b.take<float>(cnt);
    s.fbf = b.take<float>(cnt);
    if (cyclic) {
        s.z = b.take<double>(cnt);
        s.zf = b.take<float>(cnt);
        s.cv = b.take<double>(lines);
        s.sinv = b.take<double>(lines);
        s.cvf = b.take<float>(lines);
        s.sinvf = b.take<float>(lines);
    }
}

void carve_coef(Bump &b, Coef &c, size_t n, int nj1)
{
    c.AP = b.take<double>(n);
    c.AE = b.take<double>(n);
    c.AW = b.take<double>(n);
    c.AN = b.take<double>(n);
    c.AS = b.take<double>(n);
    c.ANf = b.take<float>(n);
    c.ASf = b.take<float>(n);
    c.AEf = b.take<float>(n);
    c.AWf = b.take<float>(n);
    c.awall = b.take<double>(nj1);
    c.afar = b.take<double>(nj1);
}

}  // namespace

// Tile of the radial line family: the parameters' if given; for a MIXED context
// whose Poisson sweeps run resident, two-warp groups once a line needs more than
// one warp (resident sweep on 512 x 384: 1.59 us with 2 warps x 6 elements against
// 1.86 with 4 x 3 and 1.78 with 1 x 12); else automatic (0, 0).
void radial_tile(const fvm_ctx *c, int &nw, int &m)
{
    nw = c->p.tile_r_warps;
    m = c->p.tile_r_m;
    const int n = c->NI - 1;
    if (nw || m || c->p.precision != FVM_MIXED || !c->p.poisson_resident || n <= WARP * 4) return;
    nw = 2;
    for (int mm : {1, 2, 3, 4, 6, 8})
        if (2 * WARP * mm >= n) {
            m = mm;
            return;
        }
    nw = m = 0;
}

namespace {

void carve(Bump &b, fvm_ctx *c, int nblk)
{
    Dev &d = c->d;
    const size_t n = c->n;
    const int nj1 = c->NJ + 1;
    double **geo[] = {&d.XG, &d.YG, &d.X, &d.Y, &d.XIX, &d.XIY, &d.ETX, &d.ETY, &d.DJAC, &d.Q11,
                      &d.Q12, &d.Q22, &d.DE, &d.DW, &d.DN, &d.DS, &d.THETA, &d.AREA, &d.JQ12,
                      &d.JXE, &d.JYE, &d.RJDT, &d.PJDT, &d.CNE, &d.CSE, &d.CNW, &d.CSW};
    for (auto p : geo) *p = b.take<double>(n);
    double **perj[] = {&d.UFW, &d.VFW, &d.TFW, &d.FFU, &d.FFV, &d.FFT, &d.BLOW, &d.WB};
    for (auto p : perj) *p = b.take<double>(nj1);
    double **st[] = {&d.U, &d.V, &d.P, &d.P2, &d.T, &d.U_N, &d.V_N, &d.T_N, &d.NLX, &d.NLY, &d.ADV,
                     &d.NLX_NM1, &d.NLY_NM1, &d.ADV_NM1, &d.DIFX, &d.DIFY, &d.DIFT, &d.S_U,
                     &d.S_V, &d.UE, &d.UW, &d.VN, &d.VS, &d.DIVDT, &d.SU, &d.SUV, &d.SUT,
                     &d.DD, &d.W64};
    for (auto p : st) *p = b.take<double>(n);
    d.RF = b.take<float>(n);
    d.DF = b.take<float>(n);
    d.PCD = b.take<float2>(9 * n);
    // exchange words for the largest tile (32 x 4 warps x 4 elements per line)
    d.XW = b.take<unsigned long long>(2 * size_t(c->NJ - 1) * WARP * 4 * 4);
    d.XCNT = b.take<unsigned int>(size_t(c->NJ));
    d.pctl = b.take<PCtl>(1);
    d.partial = b.take<double>(2 * size_t(nblk));
    d.coefrow = b.take<double>(8 * size_t(nj1));
    d.cflbits = b.take<unsigned long long>(1);
    d.scal = b.take<double>(16);
    carve_coef(b, d.cP, n, nj1);
    carve_coef(b, d.cUX, n, nj1);
    carve_coef(b, d.cUY, n, nj1);
    carve_coef(b, d.cTX, n, nj1);
    carve_coef(b, d.cTY, n, nj1);
    const int nr = c->NI - 1, nt = c->NJ - 1;
    int rw, rm;
    radial_tile(c, rw, rm);
    const int tw = c->p.tile_t_warps, tm = c->p.tile_t_m;
    carve_sys(b, d.sP, nt, nr, 0, rw, rm);
    carve_sys(b, d.sUX, nt, nr, 0, rw, rm);
    carve_sys(b, d.sUY, nr, nt, 1, tw, tm);
    carve_sys(b, d.sTX, nt, nr, 0, rw, rm);
    carve_sys(b, d.sTY, nr, nt, 1, tw, tm);
}

}  // namespace

int setup_allocate(fvm_ctx *c)
{
    Dev &d = c->d;
    d.NI = c->NI;
    d.NJ = c->NJ;
    d.NI1 = c->NI1;
    d.n = c->n;
    d.re = c->p.re;
    d.pe = c->p.re * c->p.pr;   // init.f90:130
    d.dt = c->p.dt;
    d.rdt = 1.0 / c->p.dt;
    d.vel_rot = c->p.vel_rot;
    d.uin = c->p.uin;
    d.vin = c->p.vin;
    d.tin = c->p.tin;
    d.t_wall = c->p.t_wall;
    d.pi = 4.0 * std::atan(1.0);
    d.resimax = c->p.resimax;
    // The FP64 sweep alternates two pressure buffers, so its residual interval is
    // even; the MIXED path checks after every refine_sweeps sweeps.  The sweep cap
    // is rounded up to a multiple of the interval in use.
    int re_ = c->p.res_every < 2 ? 2 : c->p.res_every + (c->p.res_every & 1);
    int rs_ = c->p.refine_sweeps < 1 ? 1 : c->p.refine_sweeps;
    d.res_every = re_;
    d.refine_sweeps = rs_;
    int k_ = c->p.precision == FVM_MIXED ? rs_ : re_;
    d.nswpp = ((c->p.nswpp + k_ - 1) / k_) * k_;
    d.iter_t_bug = c->p.iter_t_bug;
    d.dd_pos = c->p.dd_positional ? 1 : 0;
    d.adi_refine = c->p.adi_refine < 1 ? 1 : c->p.adi_refine;
    const int interior = (c->NI - 1) * (c->NJ - 1);
    c->nblk_res = (interior + 256 * RES_CELLS - 1) / (256 * RES_CELLS);   // residual kernels
    d.nblk_res = c->nblk_res;
    c->nblk_res64 = (interior + 256 * RES64_CELLS - 1) / (256 * RES64_CELLS);   // FP64 residual (fewer)
    d.nblk_res64 = c->nblk_res64;
    c->nblk_mres = ((c->NI - 1 + MRES_TI - 1) / MRES_TI) * ((c->NJ - 1 + MRES_TJ - 1) / MRES_TJ);
    d.nblk_mres = c->nblk_mres;
    const int nblk_partial = std::max(c->nblk_res, c->nblk_mres);
    Bump probe{nullptr};
    carve(probe, c, nblk_partial);
    c->slab_bytes = probe.off + 256;
    cudaError_t e = cudaMalloc(&c->slab, c->slab_bytes);
    if (e != cudaSuccess) {
        c->slab = nullptr;
        c->err = std::string("cudaMalloc of the context slab: ") + cudaGetErrorString(e);
        return FVM_ERR_NOMEM;
    }
    FVM_CUDA(c, cudaMemsetAsync(c->slab, 0, c->slab_bytes, c->stream));
    Bump real{c->slab};
    carve(real, c, nblk_partial);
    return FVM_OK;
}

// ---------------------------------------------------------------------------------
// GRID (grid.f90:56-114)
// ---------------------------------------------------------------------------------
__global__ void k_grid_interior(Dev d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const double *XG = d.XG, *YG = d.YG;
    d.X[IDX(i, j)] = 0.25 * (((XG[IDX(i + 1, j + 1)] + XG[IDX(i + 1, j)]) + XG[IDX(i, j + 1)]) + XG[IDX(i, j)]);
    d.Y[IDX(i, j)] = 0.25 * (((YG[IDX(i + 1, j + 1)] + YG[IDX(i + 1, j)]) + YG[IDX(i, j + 1)]) + YG[IDX(i, j)]);
}

__global__ void k_grid_edges(Dev d)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int NI = d.NI, NJ = d.NJ;
    double *X = d.X, *Y = d.Y;
    if (t >= 1 && t <= NI - 1) {   // branch-cut rows (grid.f90:66-74)
        int i = t;
        X[IDX(i, 0)] = X[IDX(i, NJ - 1)];
        Y[IDX(i, 0)] = Y[IDX(i, NJ - 1)];
        X[IDX(i, NJ)] = X[IDX(i, 1)];
        Y[IDX(i, NJ)] = Y[IDX(i, 1)];
    }
    if (t >= 1 && t <= NJ - 1) {   // wall / far-field ghosts by re-positioning (grid.f90:76-91)
        int j = t;
        double x0 = (d.XG[IDX(1, j + 1)] + d.XG[IDX(1, j)]) * 0.5;
        double y0 = (d.YG[IDX(1, j + 1)] + d.YG[IDX(1, j)]) * 0.5;
        X[IDX(0, j)] = x0 - (X[IDX(1, j)] - x0);
        Y[IDX(0, j)] = y0 - (Y[IDX(1, j)] - y0);
        double x1 = (d.XG[IDX(NI, j + 1)] + d.XG[IDX(NI, j)]) * 0.5;
        double y1 = (d.YG[IDX(NI, j + 1)] + d.YG[IDX(NI, j)]) * 0.5;
        X[IDX(NI, j)] = x1 + (x1 - X[IDX(NI - 1, j)]);
        Y[IDX(NI, j)] = y1 + (y1 - Y[IDX(NI - 1, j)]);
    }
}

__global__ void k_grid_corners(Dev d)
{   // grid.f90:94-113
    const int NI = d.NI, NJ = d.NJ;
    double *X = d.X, *Y = d.Y;
    X[IDX(0, 0)] = X[IDX(0, NJ - 1)];   Y[IDX(0, 0)] = Y[IDX(0, NJ - 1)];
    X[IDX(0, NJ)] = X[IDX(0, 1)];       Y[IDX(0, NJ)] = Y[IDX(0, 1)];
    X[IDX(NI, 0)] = X[IDX(NI, NJ - 1)]; Y[IDX(NI, 0)] = Y[IDX(NI, NJ - 1)];
    X[IDX(NI, NJ)] = X[IDX(NI, 1)];     Y[IDX(NI, NJ)] = Y[IDX(NI, 1)];
}

// ---------------------------------------------------------------------------------
// METRIC (metric.f90:18-156): derivatives at every cell incl. ghosts, Jacobian,
// inverse metrics and Q terms.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double fwd3(double a0, double a1, double a2) { return ((-(3.0 * a0)) + 4.0 * a1 - a2) / 2.0; }
__device__ __forceinline__ double bwd3(double a0, double a1, double a2) { return ((3.0 * a0 - 4.0 * a1) + a2) / 2.0; }

__device__ void derivs(const Dev &d, const double *F, int i, int j, double &dxi, double &det)
{
    const int NI = d.NI, NJ = d.NJ;
    if (i == 0) dxi = fwd3(F[IDX(0, j)], F[IDX(1, j)], F[IDX(2, j)]);
    else if (i == NI) dxi = bwd3(F[IDX(NI, j)], F[IDX(NI - 1, j)], F[IDX(NI - 2, j)]);
    else dxi = (F[IDX(i + 1, j)] - F[IDX(i - 1, j)]) / 2.0;
    if (j == 0) det = (F[IDX(i, NJ)] - F[IDX(i, NJ - 2)]) / 2.0;
    else if (j == NJ) det = (F[IDX(i, 2)] - F[IDX(i, 0)]) / 2.0;
    else det = (F[IDX(i, j + 1)] - F[IDX(i, j - 1)]) / 2.0;
}

__global__ void k_metric(Dev d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i > d.NI || j > d.NJ) return;
    double xxi, xet, yxi, yet;
    derivs(d, d.X, i, j, xxi, xet);
    derivs(d, d.Y, i, j, yxi, yet);
    int c = IDX(i, j);
    double dj = __dsub_rn(__dmul_rn(xxi, yet), __dmul_rn(yxi, xet));
    d.DJAC[c] = dj;
    double xix = yet / dj, xiy = -(xet / dj), etx = -(yxi / dj), ety = xxi / dj;
    d.XIX[c] = xix;
    d.XIY[c] = xiy;
    d.ETX[c] = etx;
    d.ETY[c] = ety;
    d.Q11[c] = __dadd_rn(__dmul_rn(xix, xix), __dmul_rn(xiy, xiy));
    d.Q12[c] = __dadd_rn(__dmul_rn(xix, etx), __dmul_rn(xiy, ety));
    d.Q22[c] = __dadd_rn(__dmul_rn(etx, etx), __dmul_rn(ety, ety));
}

// DE/DW/DN/DS (metric.f90:159-168) and products the step reuses.
__global__ void k_dcoef(Dev d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i > d.NI || j > d.NJ) return;
    int c = IDX(i, j);
    const double *J = d.DJAC;
    d.JQ12[c] = __dmul_rn(J[c], d.Q12[c]);
    d.JXE[c] = __dmul_rn(__dmul_rn(J[c], d.XIX[c]), d.ETX[c]);
    d.JYE[c] = __dmul_rn(__dmul_rn(J[c], d.XIY[c]), d.ETY[c]);
    d.RJDT[c] = (2.0 * d.re) * J[c] / d.dt;
    d.PJDT[c] = (2.0 * d.pe) * J[c] / d.dt;
    if (i < 1 || i > d.NI - 1 || j < 1 || j > d.NJ - 1) return;
    {   // diagonal weights of the cross term 0.25*(Ke(fne-fse) - Kw(fnw-fsw) + Kn(fne-fnw) - Ks(fse-fsw))
        double ke = __dmul_rn(J[IDX(i + 1, j)], d.Q12[IDX(i + 1, j)]);
        double kw = __dmul_rn(J[IDX(i - 1, j)], d.Q12[IDX(i - 1, j)]);
        double kn = __dmul_rn(J[IDX(i, j + 1)], d.Q12[IDX(i, j + 1)]);
        double ks = __dmul_rn(J[IDX(i, j - 1)], d.Q12[IDX(i, j - 1)]);
        d.CNE[c] = 0.25 * (ke + kn);
        d.CSE[c] = -(0.25 * (ke + ks));
        d.CNW[c] = -(0.25 * (kw + kn));
        d.CSW[c] = 0.25 * (kw + ks);
    }
    const double *Q1 = d.Q11, *Q2 = d.Q22;
    int e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
    d.DE[c] = 0.5 * __dadd_rn(__dmul_rn(J[c], Q1[c]), __dmul_rn(J[e], Q1[e]));
    d.DW[c] = 0.5 * __dadd_rn(__dmul_rn(J[c], Q1[c]), __dmul_rn(J[w], Q1[w]));
    d.DN[c] = 0.5 * __dadd_rn(__dmul_rn(J[c], Q2[c]), __dmul_rn(J[nn], Q2[nn]));
    d.DS[c] = 0.5 * __dadd_rn(__dmul_rn(J[c], Q2[c]), __dmul_rn(J[s], Q2[s]));
}

// THETA (init.f90:94-100): DATAN(Y/X) with the reference's quadrant fix-up.
__global__ void k_theta(Dev d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i > d.NI || j > d.NJ) return;
    int c = IDX(i, j);
    double x = d.X[c], y = d.Y[c];
    double r = sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
    double th = atan(y / x), s = asin(y / r);
    if (th >= 0.0 && s > 0.0) th = th;
    else if (th < 0.0 && s > 0.0) th = d.pi + th;
    else if (th >= 0.0 && s <= 0.0) th = d.pi + th;
    else if (th < 0.0 && s < 0.0) th = 2.0 * d.pi + th;
    d.THETA[c] = th;
}

// Wall face lengths AREA(1,J) and their sum (init.f90:120-128), wall boundary values.
__global__ void k_area(Dev d)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double sum = 0.0;
    for (int j = 1; j <= d.NJ - 1; j++) {
        double dx = d.XG[IDX(1, j + 1)] - d.XG[IDX(1, j)];
        double dy = d.YG[IDX(1, j + 1)] - d.YG[IDX(1, j)];
        double a = sqrt(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
        d.AREA[IDX(1, j)] = a;
        sum = sum + a;
    }
    d.scal[0] = sum;
}

__global__ void k_wall_values(Dev d)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > d.NJ) return;
    double th = d.THETA[IDX(0, j)];
    // bcu.f90:13, bcv.f90:13, plus the wall-normal blowing control (zero unless set)
    const double ct = cos(th), st = sin(th), b = d.BLOW[j];
    d.UFW[j] = d.vel_rot * (-st) + b * ct;
    d.VFW[j] = d.vel_rot * ct + b * st;
    d.TFW[j] = d.t_wall;                 // bct.f90:13
    // face value of J*(xi_x cos th + xi_y sin th) between the ghost and first cells:
    // the wall face flux UW(1,j) per unit blowing speed
    const int c0 = IDX(0, j), c1 = IDX(1, j);
    d.WB[j] = 0.5 * __dadd_rn(__dmul_rn(d.DJAC[c0], __dadd_rn(__dmul_rn(d.XIX[c0], ct), __dmul_rn(d.XIY[c0], st))),
                              __dmul_rn(d.DJAC[c1], __dadd_rn(__dmul_rn(d.XIX[c1], ct), __dmul_rn(d.XIY[c1], st))));
}

// Wall controls: rotation rate (VEL_ROT) and blowing speeds, then the wall values.
int setup_controls(fvm_ctx *c, double omega, const double *blow)
{
    Dev &d = c->d;
    c->p.vel_rot = omega;
    d.vel_rot = omega;
    std::vector<double> b(c->NJ + 1, 0.0);
    if (blow)
        for (int j = 1; j <= c->NJ - 1; j++) b[j] = blow[j - 1];
    FVM_CUDA(c, cudaMemcpyAsync(d.BLOW, b.data(), sizeof(double) * (c->NJ + 1), cudaMemcpyHostToDevice, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    k_wall_values<<<(c->NJ + 1 + 127) / 128, 128, 0, c->stream>>>(d);
    FVM_LAUNCH_CHECK(c);
    if (c->pgraph) cudaGraphExecDestroy(c->pgraph);
    c->pgraph = nullptr;
    return FVM_OK;
}

// ---------------------------------------------------------------------------------
// Constant coefficient sets (iter_u.f90:13-29 / 68-84, iter_p.f90:12-17) with the
// boundary folding of BCU/BCT (bcu.f90:14-16, 34-36) and BCP (bcp.f90:16-26).
// ---------------------------------------------------------------------------------
__global__ void k_coef_af(Dev d, Coef cf, const double *m1, const double *m2, double rek)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    const double *J = d.DJAC;
    int c = IDX(i, j), e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
    double ae = 0.5 * __dadd_rn(__dmul_rn(J[c], __dmul_rn(m1[c], m1[c])), __dmul_rn(J[e], __dmul_rn(m1[e], m1[e])));
    double aw = 0.5 * __dadd_rn(__dmul_rn(J[c], __dmul_rn(m1[c], m1[c])), __dmul_rn(J[w], __dmul_rn(m1[w], m1[w])));
    double an = 0.5 * __dadd_rn(__dmul_rn(J[c], __dmul_rn(m2[c], m2[c])), __dmul_rn(J[nn], __dmul_rn(m2[nn], m2[nn])));
    double as = 0.5 * __dadd_rn(__dmul_rn(J[c], __dmul_rn(m2[c], m2[c])), __dmul_rn(J[s], __dmul_rn(m2[s], m2[s])));
    double ap = (((((2.0 * rek) * J[c]) / d.dt + ae) + aw) + an) + as;
    if (i == 1) {                    // wall: AP += AW, AW = 0
        cf.awall[j] = aw;
        ap = ap + aw;
        aw = 0.0;
    }
    if (i == d.NI - 1) {             // far field: AP += AE, AE = 0
        cf.afar[j] = ae;
        ap = ap + ae;
        ae = 0.0;
    }
    cf.AE[c] = ae; cf.AW[c] = aw; cf.AN[c] = an; cf.AS[c] = as; cf.AP[c] = ap;
    cf.AEf[c] = (float)ae; cf.AWf[c] = (float)aw; cf.ANf[c] = (float)an; cf.ASf[c] = (float)as;
}

__global__ void k_coef_p(Dev d, Coef cf)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    int c = IDX(i, j);
    double ap = (((-d.DE[c]) - d.DW[c]) - d.DN[c]) - d.DS[c];
    double ae = -d.DE[c], aw = -d.DW[c], an = -d.DN[c], as = -d.DS[c];
    if (i == 1) {                    // Neumann wall: AP = AP - AW, AW = 0
        ap = ap - aw;
        aw = 0.0;
    }
    if (i == d.NI - 1) ae = 0.0;     // far field: AE = 0 (ghost enters as zero)
    cf.AE[c] = ae; cf.AW[c] = aw; cf.AN[c] = an; cf.AS[c] = as; cf.AP[c] = ap;
    cf.AEf[c] = (float)ae; cf.AWf[c] = (float)aw; cf.ANf[c] = (float)an; cf.ASf[c] = (float)as;
}

// Tridiagonal factors of one line (thread per line).  radial: unknowns i=1..NI-1 of
// row j = line+1 with a=-AW, b=AP, c=-AE.  circumferential: unknowns j=1..NJ-1 of
// column i = line+1 with a=-AS, b=AP, c=-AN, periodic (Sherman-Morrison with
// gamma = -b_1).  Recurrences as the reference's Thomas solver
// (iter_u.f90:54-63): D_e = b_e - a_e*B_{e-1}, B_e = c_e/D_e, B_0 = 0.
__global__ void k_factor(Dev d, Coef cf, LineSys s, int circ)
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
    if (circ) {
        // z = T'^{-1} u with u = (gamma, 0, ..., 0, c_n), by the same factors
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
        s.cvf[line] = (float)s.cv[line];
        s.sinvf[line] = (float)s.sinv[line];
        for (int e = 0; e < TG * M; e++) s.zf[slot(e)] = (float)s.z[slot(e)];
    }
    for (int e = 0; e < TG * M; e++) {
        size_t k = slot(e);
        s.invDf[k] = (float)s.invD[k];
        s.faf[k] = (float)s.fa[k];
        s.fbf[k] = (float)s.fb[k];
    }
}

static int build_line_sets(fvm_ctx *c)
{
    Dev &d = c->d;
    dim3 blk(128), grd((c->NI - 1 + 127) / 128, c->NJ - 1);
    k_coef_p<<<grd, blk, 0, c->stream>>>(d, d.cP);
    split_pcoef(c);
    k_coef_af<<<grd, blk, 0, c->stream>>>(d, d.cUX, d.XIX, d.ETX, d.re);
    k_coef_af<<<grd, blk, 0, c->stream>>>(d, d.cUY, d.XIY, d.ETY, d.re);
    k_coef_af<<<grd, blk, 0, c->stream>>>(d, d.cTX, d.XIX, d.ETX, d.pe);
    k_coef_af<<<grd, blk, 0, c->stream>>>(d, d.cTY, d.XIY, d.ETY, d.pe);
    FVM_LAUNCH_CHECK(c);
    return setup_factors(c);
}

// Line tiles from the parameters (0: automatic) and the factors of every line
// family in the tile's layout.  Called at setup and again when the tile changes.
int setup_factors(fvm_ctx *c)
{
    Dev &d = c->d;
    auto tile = [](LineSys &s, int nw, int m) {
        s.NW = nw > 0 ? nw : group_warps(s.n);
        s.M = m > 0 ? m : (s.n + WARP * s.NW - 1) / (WARP * s.NW);
    };
    int rw, rm;
    radial_tile(c, rw, rm);
    tile(d.sP, rw, rm);
    tile(d.sUX, rw, rm);
    tile(d.sTX, rw, rm);
    tile(d.sUY, c->p.tile_t_warps, c->p.tile_t_m);
    tile(d.sTY, c->p.tile_t_warps, c->p.tile_t_m);
    struct { Coef *cf; LineSys *s; int circ; } sets[] = {
        {&d.cP, &d.sP, 0}, {&d.cUX, &d.sUX, 0}, {&d.cUY, &d.sUY, 1}, {&d.cTX, &d.sTX, 0}, {&d.cTY, &d.sTY, 1}};
    for (auto &st : sets) {
        k_factor<<<(st.s->lines + 63) / 64, 64, 0, c->stream>>>(d, *st.cf, *st.s, st.circ);
        FVM_LAUNCH_CHECK(c);
    }
    return FVM_OK;
}

int setup_grid(fvm_ctx *c)
{
    Dev &d = c->d;
    cudaStream_t st = c->stream;
    dim3 blk(128);
    k_grid_interior<<<dim3((c->NI - 1 + 127) / 128, c->NJ - 1), blk, 0, st>>>(d);
    int m = (c->NI > c->NJ ? c->NI : c->NJ) + 1;
    k_grid_edges<<<(m + 127) / 128, 128, 0, st>>>(d);
    k_grid_corners<<<1, 1, 0, st>>>(d);
    dim3 full((c->NI + 1 + 127) / 128, c->NJ + 1);
    k_metric<<<full, blk, 0, st>>>(d);
    k_dcoef<<<full, blk, 0, st>>>(d);
    k_theta<<<full, blk, 0, st>>>(d);
    k_area<<<1, 1, 0, st>>>(d);
    k_wall_values<<<(c->NJ + 1 + 127) / 128, 128, 0, st>>>(d);
    FVM_LAUNCH_CHECK(c);
    int rc = build_line_sets(c);
    if (rc) return rc;
    // Jacobian check (metric.f90:120 prints cells with |J| < 1e-15): reject the grid
    std::vector<double> dj(c->n);
    FVM_CUDA(c, cudaMemcpyAsync(dj.data(), d.DJAC, sizeof(double) * c->n, cudaMemcpyDeviceToHost, st));
    FVM_CUDA(c, cudaStreamSynchronize(st));
    for (int k = 0; k < c->n; k++) {
        if (!(std::fabs(dj[k]) >= 1e-15)) {
            c->err = "grid has a cell with |Jacobian| < 1e-15 (or non-finite) at index " + std::to_string(k);
            return FVM_ERR_ARG;
        }
    }
    return FVM_OK;
}

// ---------------------------------------------------------------------------------
// INIT (init.f90:17-42): uniform flow + perturbation, boundary conditions applied
// with THETA still zero (the reference computes THETA only after these calls).
// ---------------------------------------------------------------------------------
__global__ void k_init_fields(Dev d, const double *du, const double *dv, int have_du, int have_dv)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i > d.NI || j > d.NJ) return;
    int c = IDX(i, j);
    bool in = i >= 1 && i <= d.NI - 1 && j >= 1 && j <= d.NJ - 1;
    d.U[c] = 1.0 + ((in && have_du) ? du[c] : 0.0);
    d.V[c] = 0.0 + ((in && have_dv) ? dv[c] : 0.0);
    d.U_N[c] = 1.0;
    d.V_N[c] = 0.0;
    d.T[c] = 0.0;
    d.T_N[c] = 0.0;
    d.P[c] = 0.0;
    d.NLX[c] = 0.0;
    d.NLY[c] = 0.0;
    d.ADV[c] = 0.0;
}

// Far-field boundary value of one field (bcu.f90:27-33): inflow Dirichlet for
// theta in [pi/2, 3pi/2], otherwise the convective outflow value built from the
// step-n field phin.  theta_zero reproduces INIT's call with THETA still zero.
__device__ __forceinline__ double farfield_value(const Dev &d, const double *phin, int j, double fin, int theta_zero)
{
    const int NI = d.NI;
    double th = theta_zero ? 0.0 : d.THETA[IDX(NI, j)];
    if (th >= 0.5 * d.pi && th <= 1.5 * d.pi) return fin;
    double a = 0.5 * (d.XIX[IDX(NI, j)] + d.XIX[IDX(NI - 1, j)]);
    double b = (0.5 * (d.ETX[IDX(NI, j)] + d.ETX[IDX(NI - 1, j)])) * 0.25;
    double dq = ((phin[IDX(NI, j + 1)] + phin[IDX(NI - 1, j + 1)]) - phin[IDX(NI, j - 1)]) - phin[IDX(NI - 1, j - 1)];
    return 0.5 * (phin[IDX(NI, j)] + phin[IDX(NI - 1, j)]) - (d.dt * d.uin) * (a * (phin[IDX(NI, j)] - phin[IDX(NI - 1, j)]) + b * dq);
}

__global__ void k_farfield(Dev d, int theta_zero)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > d.NJ - 1) return;
    d.FFU[j] = farfield_value(d, d.U_N, j, d.uin, theta_zero);
    d.FFV[j] = farfield_value(d, d.V_N, j, d.vin, theta_zero);
    d.FFT[j] = farfield_value(d, d.T_N, j, d.tin, theta_zero);
}

// Ghost columns then rows of a Dirichlet-by-ghost field with explicit wall values.
__global__ void k_bc_cols(Dev d, double *phi, const double *wallF, double wall_scalar, int use_scalar, const double *farF)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > d.NJ - 1) return;
    double w = use_scalar ? wall_scalar : wallF[j];
    phi[IDX(0, j)] = (-phi[IDX(1, j)]) + 2.0 * w;
    phi[IDX(d.NI, j)] = (-phi[IDX(d.NI - 1, j)]) + 2.0 * farF[j];
}

__global__ void k_bc_rows(Dev d, double *phi)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > d.NI) return;
    phi[IDX(i, 0)] = phi[IDX(i, d.NJ - 1)];
    phi[IDX(i, d.NJ)] = phi[IDX(i, 1)];
}

__global__ void k_copy(double *dst, const double *src, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[k];
}

int setup_init(fvm_ctx *c, const double *du, const double *dv)
{
    Dev &d = c->d;
    cudaStream_t st = c->stream;
    const size_t bytes = sizeof(double) * c->n;
    if (du) FVM_CUDA(c, cudaMemcpyAsync(d.W64, du, bytes, cudaMemcpyHostToDevice, st));
    if (dv) FVM_CUDA(c, cudaMemcpyAsync(d.DD, dv, bytes, cudaMemcpyHostToDevice, st));
    dim3 blk(128), full((c->NI + 1 + 127) / 128, c->NJ + 1);
    k_init_fields<<<full, blk, 0, st>>>(d, d.W64, d.DD, du != nullptr, dv != nullptr);
    // BCU, BCV, BCP, BCT with THETA = 0 (init.f90:33-36)
    k_farfield<<<(c->NJ + 127) / 128, 128, 0, st>>>(d, 1);
    const int gj = (c->NJ + 127) / 128, gi = (c->NI + 1 + 127) / 128;
    k_bc_cols<<<gj, 128, 0, st>>>(d, d.U, nullptr, c->p.vel_rot * (-std::sin(0.0)), 1, d.FFU);
    k_bc_rows<<<gi, 128, 0, st>>>(d, d.U);
    k_bc_cols<<<gj, 128, 0, st>>>(d, d.V, nullptr, c->p.vel_rot * std::cos(0.0), 1, d.FFV);
    k_bc_rows<<<gi, 128, 0, st>>>(d, d.V);
    k_bc_cols<<<gj, 128, 0, st>>>(d, d.T, nullptr, c->p.t_wall, 1, d.FFT);
    k_bc_rows<<<gi, 128, 0, st>>>(d, d.T);
    // P = 0 everywhere: BCP leaves it zero.
    const int nb = (c->n + 255) / 256;
    k_copy<<<nb, 256, 0, st>>>(d.U_N, d.U, c->n);
    k_copy<<<nb, 256, 0, st>>>(d.V_N, d.V, c->n);
    k_copy<<<nb, 256, 0, st>>>(d.T_N, d.T, c->n);
    FVM_LAUNCH_CHECK(c);
    FVM_CUDA(c, cudaStreamSynchronize(st));
    c->rtime = 0.0;
    c->niter_time = 0;
    return FVM_OK;
}

}  // namespace fvm
