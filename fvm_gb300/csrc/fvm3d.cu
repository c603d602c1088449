// fvm3d.cu -- the 3-D LES time step of the cylinder solver on one GB300
// (reference: LES/v2.3_LES-Reynolds stresses/, main.f90:33-147), FP64.
//
// GPU order, restated by the CPU oracle's O3_GPU mode: every line sweep is
// red-black over lines (a line's colour is the parity of the sum of its two
// transverse indices; with NJ-1 and NK-1 even the colouring is consistent across
// the periodic wraps), neighbours across the branch cut and the spanwise period
// are read through index wrap, and the J and K lines of the predictor are solved
// as cyclic systems.  Ghost cells are refreshed exactly where the reference calls
// its BC routines (BCU/BCT before every predictor sweep, BCP before every Poisson
// sweep), so cross terms see the same lagged ghosts.  The reference's single-rank
// MPI_X is a periodic copy (halo kernels: J planes, then K planes).
//
// Line solves reuse the group solver of the 2-D path (precomputed LU factors in
// chunk-interleaved layout, warp scans of affine maps, Sherman-Morrison for the
// cyclic lines).
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "fvm_df.cuh"
#include "fvm_internal.cuh"
#include "../../include/fvm3d.h"

namespace fvm {
// warp shuffles of a double-float value (the group line solver's scans)
template <>
__device__ __forceinline__ dd shfl_up<dd>(dd v, int s)
{
    return dd(__shfl_up_sync(0xffffffffu, v.hi, s), __shfl_up_sync(0xffffffffu, v.lo, s));
}
template <>
__device__ __forceinline__ dd shfl_down<dd>(dd v, int s)
{
    return dd(__shfl_down_sync(0xffffffffu, v.hi, s), __shfl_down_sync(0xffffffffu, v.lo, s));
}
}  // namespace fvm

namespace f3 {

using fvm::dd;
using fvm::ld;
using fvm::LineSys;
using fvm::scale2;
using fvm::to_d;
using fvm::PCtl;
using fvm::WARP;

// Seven-point coefficient set with the wall / far-field folding applied; the raw
// folded coefficients per (j,k) for the boundary source terms.
struct Coef3 {
    double *AP, *AE, *AW, *AN, *AS, *AT, *AB;
    double *awall, *afar;   // (NJ+1)*(NK+1)
};

// Double-float copies of a predictor set's line factors (mixed path).
struct LineDD {
    dd *invD, *fa, *fb, *z, *cv, *sinv;
};

struct D3 {
    int NI, NJ, NK, NI1, NJ1, n, nblk;
    double re, pe, dt, rdt, tin, t_wall, pi, resimax, ref_a;
    double r2re_dt, r2pe_dt;   // 2 Re / dt and 2 Pe / dt (double-float AF right-hand sides)
    // Mixed path: the arrays read by the double-float kernels have (hi, lo) float
    // pair shadows at the constant element offset sh (dfl = 1); see carve().
    long long sh;
    int dfl;
    int nswpp, res_every, les_zavg, thermal, refine_sweeps;
    // geometry
    double *XG, *YG, *ZG, *X, *Y, *Z;
    double *XIX, *XIY, *XIZ, *ETX, *ETY, *ETZ, *ZTX, *ZTY, *ZTZ, *DJAC;
    double *Q11, *Q12, *Q13, *Q22, *Q23, *Q33;
    double *JQ12, *JQ13, *JQ23;   // Q12*DJAC, Q13*DJAC, Q23*DJAC
    // The twelve-term cross derivatives as weights of the 12 edge neighbours (see
    // k3_cw): CW for DIF_DIAGONAL / ITER_P, CWA[s] for the AF split s of ITER_U/T.
    double *CW[12], *CWA[3][12];
    double *DE, *DW, *DN, *DS, *DT, *DB, *THETA, *AREA1, *AREA2, *FW;
    double *MD[9];          // metric derivatives (scratch of the setup)
    // state
    double *U, *V, *W, *P, *T, *U_N, *V_N, *W_N, *T_N;
    double *NLX, *NLY, *NLZ, *ADV, *NLX_NM1, *NLY_NM1, *NLZ_NM1, *ADV_NM1;
    double *DIFX, *DIFY, *DIFZ, *DIFT, *S_U, *S_V, *S_W;
    double *U1, *U2, *U3, *UE, *UW, *VN, *VS, *WT, *WB, *DIVDT, *SU;
    double *FFU, *FFV, *FFW, *FFT;   // far-field boundary values per (j,k) (step)
    // LES
    double *L[9], *DTD[3], *MAG, *UH, *VH, *WH, *TH, *MAGH, *LM, *MM, *EV, *EC, *CZ;
    // coefficient sets: [0..2] velocity splits, [3..5] temperature splits, [6] Poisson
    Coef3 cf[7];
    LineSys sys[7];
    LineDD sysd[6];   // mixed path: the factors of the six predictor sets as (hi, lo) pairs
    // MIXED Poisson: FP32 residual and correction, FP32 copies of the transverse
    // couplings of the Poisson set
    // (the Poisson operator is symmetric: AS(j) = AN(j-1) and AB(k) = AT(k-1), the
    // south and bottom couplings are read as the neighbours' north and top ones)
    float *RF, *DF, *ANf, *ATf;
    // SGS model: two banks of 12 arrays for the separable test filters
    double *FB;
    // reductions
    PCtl *pctl;
    double *partial;        // 4 per block
    double *scal;           // [0] C_s, [1] C_t, [2] reference pressure, [3..] coefficients
    unsigned long long *cflbits;
    double *wall;           // 8 per (j,k) and triangle
};

#define ID3(i, j, k) ((i) + d.NI1 * ((j) + d.NJ1 * (k)))
#define JK(j, k) ((j) + d.NJ1 * (k))

__device__ __forceinline__ int jw(const D3 &d, int j) { return j == 0 ? d.NJ - 1 : (j == d.NJ ? 1 : j); }
__device__ __forceinline__ int kw(const D3 &d, int k) { return k == 0 ? d.NK - 1 : (k == d.NK ? 1 : k); }

// Thread -> cell of a 3-D launch over (i0..i1) x (j0..j1) x (k0..k1).
#define CELL3(i0, i1, j0, j1, k0, k1)                                                               \
    const int i = blockIdx.x * blockDim.x + threadIdx.x + (i0);                                     \
    const int j = blockIdx.y * blockDim.y + threadIdx.y + (j0);                                     \
    const int k = blockIdx.z + (k0);                                                                \
    if (i > (i1) || j > (j1) || k > (k1)) return;

// The (hi, lo) shadow of an array of the shadowed group (mixed path only).
__device__ __forceinline__ float2 *shadow(const D3 &d, const double *p)
{
    return reinterpret_cast<float2 *>(const_cast<double *>(p) + d.sh);
}
// Element c of a shadowed array in arithmetic type T: the double itself (FP64 path)
// or its shadow pair (mixed path; no split on the load).
template <class T>
__device__ __forceinline__ T lds(const D3 &d, const double *p, int c);
template <>
__device__ __forceinline__ double lds<double>(const D3 &, const double *p, int c) { return p[c]; }
template <>
__device__ __forceinline__ dd lds<dd>(const D3 &d, const double *p, int c)
{
    const float2 v = shadow(d, p)[c];
    return dd(v.x, v.y);
}
// Store into a shadowed array: the double, and in the mixed path its shadow too.
__device__ __forceinline__ void sts(const D3 &, double *p, int c, double v) { p[c] = v; }
__device__ __forceinline__ void sts(const D3 &d, double *p, int c, dd v)
{
    p[c] = fvm::dd_join(v);
    shadow(d, p)[c] = make_float2(v.hi, v.lo);
}

// ---------------------------------------------------------------------------------
// Periodic copy of MPI_X (mpi_x.f90:25-51): J planes for every K, then K planes for
// every J, as one launch (k3_halo).  Up to 16 arrays per launch.
// ---------------------------------------------------------------------------------
struct Arrs {
    double *a[16];
    int n;
};

// Both copies in one launch: the final value of every ghost (j in {0, NJ} or k in
// {0, NK}) is the interior value at the wrapped indices, which the J-then-K pair
// produces; grid y < NK+1 takes the J ghosts of plane k = y, the rest the K ghosts
// of row j = y - NK - 1 (the corner ghosts are written twice with the same value).
__global__ void k3_halo(D3 d, Arrs A)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (i > d.NI) return;
    if (r <= d.NK) {
        const int k = r, ks = kw(d, k);
        for (int q = 0; q < A.n; q++) {
            double *a = A.a[q];
            a[ID3(i, 0, k)] = a[ID3(i, d.NJ - 1, ks)];
            a[ID3(i, d.NJ, k)] = a[ID3(i, 1, ks)];
        }
    } else {
        const int j = r - d.NK - 1, js = jw(d, j);
        for (int q = 0; q < A.n; q++) {
            double *a = A.a[q];
            a[ID3(i, j, 0)] = a[ID3(i, js, d.NK - 1)];
            a[ID3(i, j, d.NK)] = a[ID3(i, js, 1)];
        }
    }
}

// The shadows of up to 16 shadowed arrays over the whole array (mixed path).
__global__ void k3_shadow(D3 d, Arrs A)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    for (int q = 0; q < A.n; q++) {
        const dd v = fvm::dd_split(A.a[q][c]);
        shadow(d, A.a[q])[c] = make_float2(v.hi, v.lo);
    }
}

// ---------------------------------------------------------------------------------
// GRID (grid.f90:75-320)
// ---------------------------------------------------------------------------------
__global__ void k3_centres(D3 d)
{
    CELL3(0, d.NI, 0, d.NJ, 0, d.NK)
    double *C[3] = {d.X, d.Y, d.Z};
    const double *G[3] = {d.XG, d.YG, d.ZG};
    const bool ii = i >= 1 && i <= d.NI - 1, jj = j >= 1 && j <= d.NJ - 1, kk = k >= 1 && k <= d.NK - 1;
    for (int q = 0; q < 3; q++) {
        const double *g = G[q];
        if (ii && jj && kk)
            C[q][ID3(i, j, k)] = 0.125 * (((((((g[ID3(i + 1, j + 1, k)] + g[ID3(i + 1, j, k)]) + g[ID3(i, j + 1, k)]) +
                                              g[ID3(i, j, k)]) + g[ID3(i + 1, j + 1, k + 1)]) + g[ID3(i + 1, j, k + 1)]) +
                                           g[ID3(i, j + 1, k + 1)]) + g[ID3(i, j, k + 1)]);
    }
}

// Boundary faces (face centre mirrored across the face); reads interior centres.
__global__ void k3_faces(D3 d)
{
    CELL3(0, d.NI, 0, d.NJ, 0, d.NK)
    double *C[3] = {d.X, d.Y, d.Z};
    const double *G[3] = {d.XG, d.YG, d.ZG};
    const bool ii = i >= 1 && i <= d.NI - 1, jj = j >= 1 && j <= d.NJ - 1, kk = k >= 1 && k <= d.NK - 1;
    for (int q = 0; q < 3; q++) {
        double *A = C[q];
        const double *g = G[q];
        const int c = ID3(i, j, k);
        if (i == 0 && jj && kk) {
            double f = 0.25 * (((g[ID3(1, j + 1, k)] + g[ID3(1, j, k)]) + g[ID3(1, j + 1, k + 1)]) + g[ID3(1, j, k + 1)]);
            A[c] = f - (A[ID3(1, j, k)] - f);
        } else if (i == d.NI && jj && kk) {
            double f = 0.25 * (((g[ID3(i, j + 1, k)] + g[ID3(i, j, k)]) + g[ID3(i, j + 1, k + 1)]) + g[ID3(i, j, k + 1)]);
            A[c] = f + (f - A[ID3(i - 1, j, k)]);
        } else if (j == 0 && ii && kk) {
            double f = 0.25 * (((g[ID3(i + 1, 1, k + 1)] + g[ID3(i + 1, 1, k)]) + g[ID3(i, 1, k + 1)]) + g[ID3(i, 1, k)]);
            A[c] = f - (A[ID3(i, 1, k)] - f);
        } else if (j == d.NJ && ii && kk) {
            double f = 0.25 * (((g[ID3(i + 1, j, k + 1)] + g[ID3(i + 1, j, k)]) + g[ID3(i, j, k + 1)]) + g[ID3(i, j, k)]);
            A[c] = f - (A[ID3(i, j - 1, k)] - f);
        } else if (k == 0 && ii && jj) {
            double f = 0.25 * (((g[ID3(i, j, 1)] + g[ID3(i + 1, j, 1)]) + g[ID3(i + 1, j + 1, 1)]) + g[ID3(i, j + 1, 1)]);
            A[c] = f - (A[ID3(i, j, 1)] - f);
        } else if (k == d.NK && ii && jj) {
            double f = 0.25 * (((g[ID3(i, j, k)] + g[ID3(i + 1, j, k)]) + g[ID3(i + 1, j + 1, k)]) + g[ID3(i, j + 1, k)]);
            A[c] = f + (f - A[ID3(i, j, k - 1)]);
        }
    }
}

// Spanwise end planes after the periodic copy (grid.f90:261-320): x, y copied from
// the adjacent plane, z mirrored across the end face (edges and corners copied).
__global__ void k3_kplanes_xy_zin(D3 d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, side = blockIdx.z;
    if (i > d.NI || j > d.NJ) return;
    const int k = side ? d.NK : 0, kin = side ? d.NK - 1 : 1;
    d.X[ID3(i, j, k)] = d.X[ID3(i, j, kin)];
    d.Y[ID3(i, j, k)] = d.Y[ID3(i, j, kin)];
    if (i >= 1 && i <= d.NI - 1 && j >= 1 && j <= d.NJ - 1) {
        const double *g = d.ZG;
        double f = side ? 0.25 * (((g[ID3(i, j, k)] + g[ID3(i + 1, j, k)]) + g[ID3(i + 1, j + 1, k)]) + g[ID3(i, j + 1, k)])
                        : 0.25 * (((g[ID3(i, j, 1)] + g[ID3(i + 1, j, 1)]) + g[ID3(i + 1, j + 1, 1)]) + g[ID3(i, j + 1, 1)]);
        d.Z[ID3(i, j, k)] = side ? f + (f - d.Z[ID3(i, j, kin)]) : f - (d.Z[ID3(i, j, kin)] - f);
    }
}

__global__ void k3_kplanes_zedge(D3 d)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x, side = blockIdx.y;
    const int k = side ? d.NK : 0, NI = d.NI, NJ = d.NJ;
    double *Z = d.Z;
    if (t >= 1 && t <= NJ - 1) {
        Z[ID3(0, t, k)] = Z[ID3(1, t, k)];
        Z[ID3(NI, t, k)] = Z[ID3(NI - 1, t, k)];
    }
    if (t >= 1 && t <= NI - 1) {
        Z[ID3(t, 0, k)] = Z[ID3(t, 1, k)];
        Z[ID3(t, NJ, k)] = Z[ID3(t, NJ - 1, k)];
    }
}

__global__ void k3_kplanes_zcorner(D3 d)
{
    const int side = threadIdx.x;
    if (side > 1) return;
    const int k = side ? d.NK : 0, NI = d.NI, NJ = d.NJ;
    double *Z = d.Z;
    Z[ID3(0, 0, k)] = Z[ID3(1, 1, k)];
    Z[ID3(NI, 0, k)] = Z[ID3(NI - 1, 1, k)];
    Z[ID3(NI, NJ, k)] = Z[ID3(NI - 1, NJ - 1, k)];
    Z[ID3(0, NJ, k)] = Z[ID3(1, NJ - 1, k)];
}

// ---------------------------------------------------------------------------------
// METRIC (metric.f90:33-520)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double dref(const D3 &d, const double *A, int i, int j, int k, int dir)
{
    const int hi = dir == 0 ? d.NI : (dir == 1 ? d.NJ : d.NK);
    const int q = dir == 0 ? i : (dir == 1 ? j : k);
    const int si = dir == 0, sj = dir == 1, sk = dir == 2;
#define AT3(s) A[ID3(i + (s) * si, j + (s) * sj, k + (s) * sk)]
    if (q == 0) return __ddiv_rn(__dadd_rn(__dadd_rn(-3.0 * AT3(0), 4.0 * AT3(1)), -AT3(2)), 2.0);
    if (q == hi) return __ddiv_rn(__dadd_rn(__dadd_rn(3.0 * AT3(0), -4.0 * AT3(-1)), AT3(-2)), 2.0);
    return 0.5 * (AT3(1) - AT3(-1));
#undef AT3
}

__global__ void k3_derivs(D3 d)
{
    CELL3(0, d.NI, 0, d.NJ, 0, d.NK)
    const double *C[3] = {d.X, d.Y, d.Z};
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) d.MD[3 * a + b][ID3(i, j, k)] = dref(d, C[a], i, j, k, b);
}

__global__ void k3_jacobian(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const double XXI = d.MD[0][c], XET = d.MD[1][c], XZT = d.MD[2][c], YXI = d.MD[3][c], YET = d.MD[4][c],
                 YZT = d.MD[5][c], ZXI = d.MD[6][c], ZET = d.MD[7][c], ZZT = d.MD[8][c];
#define M_(a, b) __dmul_rn(a, b)
#define S_(a, b) __dsub_rn(a, b)
    double J = __dadd_rn(S_(M_(XXI, S_(M_(YET, ZZT), M_(YZT, ZET))), M_(YXI, S_(M_(XET, ZZT), M_(ZET, XZT)))),
                         M_(ZXI, S_(M_(XET, YZT), M_(XZT, YET))));
    d.DJAC[c] = J;
    d.XIX[c] = __ddiv_rn(S_(M_(YET, ZZT), M_(YZT, ZET)), J);
    d.XIY[c] = __ddiv_rn(S_(M_(ZET, XZT), M_(ZZT, XET)), J);
    d.XIZ[c] = __ddiv_rn(S_(M_(XET, YZT), M_(XZT, YET)), J);
    d.ETX[c] = __ddiv_rn(S_(M_(YZT, ZXI), M_(YXI, ZZT)), J);
    d.ETY[c] = __ddiv_rn(S_(M_(ZZT, XXI), M_(ZXI, XZT)), J);
    d.ETZ[c] = __ddiv_rn(S_(M_(XZT, YXI), M_(XXI, YZT)), J);
    d.ZTX[c] = __ddiv_rn(S_(M_(YXI, ZET), M_(YET, ZXI)), J);
    d.ZTY[c] = __ddiv_rn(S_(M_(ZXI, XET), M_(ZET, XXI)), J);
    d.ZTZ[c] = __ddiv_rn(S_(M_(XXI, YET), M_(XET, YXI)), J);
#undef M_
#undef S_
}

__device__ __forceinline__ double dot3(double a1, double b1, double a2, double b2, double a3, double b3)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(a1, b1), __dmul_rn(a2, b2)), __dmul_rn(a3, b3));
}

__global__ void k3_q(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const double xx = d.XIX[c], xy = d.XIY[c], xz = d.XIZ[c], ex = d.ETX[c], ey = d.ETY[c], ez = d.ETZ[c],
                 zx = d.ZTX[c], zy = d.ZTY[c], zz = d.ZTZ[c];
    d.Q11[c] = dot3(xx, xx, xy, xy, xz, xz);
    d.Q12[c] = dot3(xx, ex, xy, ey, xz, ez);
    d.Q13[c] = dot3(zx, xx, zy, xy, zz, xz);
    d.Q22[c] = dot3(ex, ex, ey, ey, ez, ez);
    d.Q23[c] = dot3(ex, zx, ey, zy, ez, zz);
    d.Q33[c] = dot3(zx, zx, zy, zy, zz, zz);
    d.FW[c] = pow(d.DJAC[c], 1.0 / 3.0);
    d.JQ12[c] = d.Q12[c] * d.DJAC[c];
    d.JQ13[c] = d.Q13[c] * d.DJAC[c];
    d.JQ23[c] = d.Q23[c] * d.DJAC[c];
}

__global__ void k3_dcoef(D3 d)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const double *J = d.DJAC;
    const int c = ID3(i, j, k);
    auto h = [&](const double *Q, int o) { return 0.5 * __dadd_rn(__dmul_rn(J[c], Q[c]), __dmul_rn(J[o], Q[o])); };
    d.DE[c] = h(d.Q11, ID3(i + 1, j, k));
    d.DW[c] = h(d.Q11, ID3(i - 1, j, k));
    d.DN[c] = h(d.Q22, ID3(i, j + 1, k));
    d.DS[c] = h(d.Q22, ID3(i, j - 1, k));
    d.DT[c] = h(d.Q33, ID3(i, j, k + 1));
    d.DB[c] = h(d.Q33, ID3(i, j, k - 1));
}

// THETA over the whole array (init.f90:155-168)
__global__ void k3_theta(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const double X = d.X[c], Y = d.Y[c];
    double R = sqrt(__dadd_rn(__dmul_rn(X, X), __dmul_rn(Y, Y)));
    double th = atan(Y / X);
    double s = asin(Y / R);
    if (th >= 0.0 && s > 0.0) th = th;
    else if (th < 0.0 && s > 0.0) th = d.pi + th;
    else if (th >= 0.0 && s <= 0.0) th = d.pi + th;
    else if (th < 0.0 && s < 0.0) th = 2.0 * d.pi + th;
    d.THETA[c] = th;
}

// Wall face triangles at I=1 (init.f90:172-190)
__global__ void k3_areas(D3 d)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (j > d.NJ - 1 || k > d.NK - 1) return;
    const int i = 1;
    const double *XG = d.XG, *YG = d.YG, *ZG = d.ZG;
    auto len = [&](int a, int b) {
        double dx = XG[a] - XG[b], dy = YG[a] - YG[b], dz = ZG[a] - ZG[b];
        return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    };
    const int p00 = ID3(i, j, k), p10 = ID3(i, j + 1, k), p01 = ID3(i, j, k + 1), p11 = ID3(i, j + 1, k + 1);
    double L1 = len(p10, p00), L2 = len(p01, p00), L3 = len(p10, p01);
    double TH1 = acos(__ddiv_rn(__dsub_rn(__dsub_rn(L3 * L3, L2 * L2), L1 * L1), __dmul_rn(-2.0 * L1, L2)));
    d.AREA1[p00] = __dmul_rn(__dmul_rn(0.5 * L1, L2), sin(TH1));
    L1 = len(p11, p10);
    L2 = len(p11, p01);
    TH1 = acos(__ddiv_rn(__dsub_rn(__dsub_rn(L3 * L3, L2 * L2), L1 * L1), __dmul_rn(-2.0 * L1, L2)));
    d.AREA2[p00] = __dmul_rn(__dmul_rn(0.5 * L1, L2), sin(TH1));
}

}  // namespace f3

namespace f3 {

// ---------------------------------------------------------------------------------
// Constant coefficient sets with the BC folding (iter_u.f90:23-42 per split,
// bcu.f90:18-24, 41-44; iter_p.f90:14-26, bcp.f90:24-32)
// ---------------------------------------------------------------------------------
__global__ void k3_coef_af(D3 d, Coef3 cf, int split, double rek)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const double *J = d.DJAC;
    const double *m1 = split == 0 ? d.XIX : (split == 1 ? d.XIY : d.XIZ);
    const double *m2 = split == 0 ? d.ETX : (split == 1 ? d.ETY : d.ETZ);
    const double *m3 = split == 0 ? d.ZTX : (split == 1 ? d.ZTY : d.ZTZ);
    const int c = ID3(i, j, k);
    auto h = [&](const double *m, int o) {
        return 0.5 * __dadd_rn(__dmul_rn(J[c], __dmul_rn(m[c], m[c])), __dmul_rn(J[o], __dmul_rn(m[o], m[o])));
    };
    double ae = h(m1, ID3(i + 1, j, k)), aw = h(m1, ID3(i - 1, j, k)), an = h(m2, ID3(i, j + 1, k)),
           as = h(m2, ID3(i, j - 1, k)), at = h(m3, ID3(i, j, k + 1)), ab = h(m3, ID3(i, j, k - 1));
    double ap = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__ddiv_rn(__dmul_rn(2.0 * rek, J[c]), d.dt),
                                                                              ae), aw), an), as), at), ab);
    if (i == 1) {
        cf.awall[JK(j, k)] = aw;
        ap = __dadd_rn(ap, aw);
        aw = 0.0;
    }
    if (i == d.NI - 1) {
        cf.afar[JK(j, k)] = ae;
        ap = __dadd_rn(ap, ae);
        ae = 0.0;
    }
    cf.AP[c] = ap; cf.AE[c] = ae; cf.AW[c] = aw; cf.AN[c] = an; cf.AS[c] = as; cf.AT[c] = at; cf.AB[c] = ab;
}

__global__ void k3_coef_p(D3 d, Coef3 cf)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    double ap = (((((-d.DE[c]) - d.DW[c]) - d.DN[c]) - d.DS[c]) - d.DT[c]) - d.DB[c];
    double ae = -d.DE[c], aw = -d.DW[c];
    if (i == 1) {
        ap = ap - aw;
        aw = 0.0;
    }
    if (i == d.NI - 1) ae = 0.0;
    cf.AP[c] = ap; cf.AE[c] = ae; cf.AW[c] = aw;
    cf.AN[c] = -d.DN[c]; cf.AS[c] = -d.DS[c]; cf.AT[c] = -d.DT[c]; cf.AB[c] = -d.DB[c];
}

// Weights of the 12 edge neighbours of an interior cell for products A12..A32 given
// by prod(pair, cell): pair 0 A12 (the I direction of the (i,j) pair), 1 A21,
// 2 A13, 3 A31, 4 A23, 5 A32.  set < 0: DIF_DIAGONAL / ITER_P (A_xy = J*Q_xy,
// symmetric); set = s: AF split s, A_xy = (J m_x) m_y with the split's metrics.
__global__ void k3_cw(D3 d, int set)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    const double *J = d.DJAC;
    const double *m[3] = {set == 0 ? d.XIX : (set == 1 ? d.XIY : d.XIZ), set == 0 ? d.ETX : (set == 1 ? d.ETY : d.ETZ),
                          set == 0 ? d.ZTX : (set == 1 ? d.ZTY : d.ZTZ)};
    auto prod = [&](int x, int y, int cell) {   // A_xy at cell (x, y in 0..2)
        if (set < 0) {
            const int q = x + y;   // 1: Q12, 2: Q13, 3: Q23
            return (q == 1 ? d.JQ12 : (q == 2 ? d.JQ13 : d.JQ23))[cell];
        }
        return (J[cell] * m[x][cell]) * m[y][cell];
    };
    const int sj = d.NI1, sk = d.NI1 * d.NJ1;
    const int st[3] = {1, sj, sk};
    const int px[3] = {0, 0, 1}, py[3] = {1, 2, 2};   // the three pairs (i,j), (i,k), (j,k)
    double *const *W = set < 0 ? d.CW : d.CWA[set];
#pragma unroll
    for (int pr = 0; pr < 3; pr++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int a = (q & 2) ? -1 : 1, b = (q & 1) ? -1 : 1, x = px[pr], y = py[pr];
            const double w = prod(x, y, c + a * st[x]) + prod(y, x, c + b * st[y]);
            W[4 * pr + q][c] = (0.25 * (double)(a * b)) * w;
        }
}

// Line families: 0 = I lines (transverse j,k), 1 = J lines (i,k), 2 = K lines (i,j).
struct Fam {
    int n, lines;
};

__host__ __device__ inline Fam family(int fam, int NI, int NJ, int NK)
{
    if (fam == 0) return {NI - 1, (NJ - 1) * (NK - 1)};
    if (fam == 1) return {NJ - 1, (NI - 1) * (NK - 1)};
    return {NK - 1, (NI - 1) * (NJ - 1)};
}

// Cell of element e of line L of a family.
__device__ __forceinline__ int line_cell(const D3 &d, int fam, int L, int e)
{
    if (fam == 0) return ID3(e + 1, L % (d.NJ - 1) + 1, L / (d.NJ - 1) + 1);
    if (fam == 1) return ID3(L % (d.NI - 1) + 1, e + 1, L / (d.NI - 1) + 1);
    return ID3(L % (d.NI - 1) + 1, L / (d.NI - 1) + 1, e + 1);
}

// LU factors (and the Sherman-Morrison vector of cyclic lines) of one family, in
// the group solver's chunk-interleaved layout (as k_factor of the 2-D path).
__global__ void k3_factor(D3 d, Coef3 cf, LineSys s, int fam, int cyc)
{
    const int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= s.lines) return;
    const int n = s.n, M = s.M, TG = WARP * s.NW;
    const size_t base = size_t(L) * TG * M;
    auto slot = [&](int e) { return base + size_t(e % M) * TG + (e / M); };
    auto lo = [&](int c) { return fam == 0 ? cf.AW[c] : (fam == 1 ? cf.AS[c] : cf.AB[c]); };
    auto hi = [&](int c) { return fam == 0 ? cf.AE[c] : (fam == 1 ? cf.AN[c] : cf.AT[c]); };
    double gamma = 0.0, a1 = 0.0, cn = 0.0;
    if (cyc) {
        gamma = -cf.AP[line_cell(d, fam, L, 0)];
        a1 = -lo(line_cell(d, fam, L, 0));
        cn = -hi(line_cell(d, fam, L, n - 1));
    }
    double Bprev = 0.0;
    for (int e = 0; e < n; e++) {
        const int c = line_cell(d, fam, L, e);
        double a = -lo(c), b = cf.AP[c], cc = -hi(c);
        if (cyc && e == 0) { a = 0.0; b = b - gamma; }
        if (cyc && e == n - 1) { b = b - a1 * cn / gamma; cc = 0.0; }
        if (!cyc && e == 0) a = 0.0;
        if (!cyc && e == n - 1) cc = 0.0;
        double D = b - a * Bprev;
        double B = cc / D;
        size_t q = slot(e);
        s.invD[q] = 1.0 / D;
        s.fa[q] = -a / D;
        s.fb[q] = -B;
        Bprev = B;
    }
    for (int e = n; e < TG * M; e++) {
        size_t q = slot(e);
        s.invD[q] = 0.0;
        s.fa[q] = 0.0;
        s.fb[q] = 0.0;
    }
    if (cyc) {
        double y = 0.0;
        for (int e = 0; e < n; e++) {
            double u = (e == 0) ? gamma : (e == n - 1 ? cn : 0.0);
            size_t q = slot(e);
            y = s.fa[q] * y + s.invD[q] * u;
            s.z[q] = y;
        }
        double x = 0.0;
        for (int e = n - 1; e >= 0; e--) {
            size_t q = slot(e);
            x = s.z[q] + s.fb[q] * x;
            s.z[q] = x;
        }
        for (int e = n; e < TG * M; e++) s.z[slot(e)] = 0.0;
        double cv = a1 / gamma;
        s.cv[L] = cv;
        s.sinv[L] = 1.0 / (1.0 + s.z[slot(0)] + cv * s.z[slot(n - 1)]);
    }
    for (int e = 0; e < TG * M; e++) {
        size_t q = slot(e);
        s.invDf[q] = (float)s.invD[q];
        s.faf[q] = (float)s.fa[q];
        s.fbf[q] = (float)s.fb[q];
        if (cyc) s.zf[q] = (float)s.z[q];
    }
    if (cyc) {
        s.cvf[L] = (float)s.cv[L];
        s.sinvf[L] = (float)s.sinv[L];
    }
}

// ---------------------------------------------------------------------------------
// Red-black line sweep of one family (GPU order).  Colour c takes the lines whose
// transverse index sum has parity c; the couplings to the other lines are read
// through periodic wrap; J and K lines are cyclic.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool colour_line(const D3 &d, int fam, int colour, int gl, int &L)
{
    if (fam == 0) {   // transverse (j,k): per k, (NJ-1)/2 lines
        const int h = (d.NJ - 1) / 2, k = gl / h + 1;
        if (k > d.NK - 1) return false;
        const int j = (((1 + k) & 1) == colour ? 1 : 2) + 2 * (gl % h);
        L = (j - 1) + (d.NJ - 1) * (k - 1);
        return true;
    }
    if (fam == 1) {   // transverse (i,k): per i, (NK-1)/2 lines
        const int h = (d.NK - 1) / 2, i = gl / h + 1;
        if (i > d.NI - 1) return false;
        const int k = (((i + 1) & 1) == colour ? 1 : 2) + 2 * (gl % h);
        L = (i - 1) + (d.NI - 1) * (k - 1);
        return true;
    }
    const int h = (d.NJ - 1) / 2, i = gl / h + 1;   // transverse (i,j)
    if (i > d.NI - 1) return false;
    const int j = (((i + 1) & 1) == colour ? 1 : 2) + 2 * (gl % h);
    L = (i - 1) + (d.NI - 1) * (j - 1);
    return true;
}

// Cell index of element 0 of line L, the element stride, and the offsets of the
// four transverse neighbours (periodic wrap applied once per line).
struct LineGeo {
    int base, stride, o1, o2, o3, o4;
};

template <int FAM>
__device__ __forceinline__ LineGeo line_geo(const D3 &d, int L)
{
    const int sj = d.NI1, sk = d.NI1 * d.NJ1;
    LineGeo g;
    if (FAM == 0) {   // I line (j, k): couplings N, S, T, B
        const int j = L % (d.NJ - 1) + 1, k = L / (d.NJ - 1) + 1;
        g.base = ID3(1, j, k);
        g.stride = 1;
        g.o1 = (jw(d, j + 1) - j) * sj;
        g.o2 = (jw(d, j - 1) - j) * sj;
        g.o3 = (kw(d, k + 1) - k) * sk;
        g.o4 = (kw(d, k - 1) - k) * sk;
    } else if (FAM == 1) {   // J line (i, k): couplings E, W, T, B
        const int i = L % (d.NI - 1) + 1, k = L / (d.NI - 1) + 1;
        g.base = ID3(i, 1, k);
        g.stride = sj;
        g.o1 = 1;
        g.o2 = -1;
        g.o3 = (kw(d, k + 1) - k) * sk;
        g.o4 = (kw(d, k - 1) - k) * sk;
    } else {   // K line (i, j): couplings E, W, N, S
        const int i = L % (d.NI - 1) + 1, j = L / (d.NI - 1) + 1;
        g.base = ID3(i, j, 1);
        g.stride = sk;
        g.o1 = 1;
        g.o2 = -1;
        g.o3 = (jw(d, j + 1) - j) * sj;
        g.o4 = (jw(d, j - 1) - j) * sj;
    }
    return g;
}

// The four coupling coefficients of a family in the order of its neighbour offsets.
template <int FAM>
__device__ __forceinline__ void couple_coefs(const Coef3 &cf, const double *&c1, const double *&c2,
                                             const double *&c3, const double *&c4)
{
    c1 = FAM == 0 ? cf.AN : cf.AE;
    c2 = FAM == 0 ? cf.AS : cf.AW;
    c3 = FAM == 2 ? cf.AN : cf.AT;
    c4 = FAM == 2 ? cf.AS : cf.AB;
}

// T: double (FP64 path, every set) or dd (mixed path, the predictor sets 0..5, whose
// couplings and phi are read through their shadows and factors from sd; phi is
// stored with its shadow, so the second colour reads the first colour's values).
template <int M, int NW, int FAM, class T = double>
__global__ void __launch_bounds__(128) k3_line(D3 d, LineSys s, Coef3 cf, const double *SU, double *phi, int colour,
                                               const PCtl *stop, LineDD sd)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ T sm[G][TG * M + M * NW + 1];
    __shared__ T xch[G][2 * NW];
    const int ended = stop ? stop->done : 0;   // the Poisson loop has ended (tested after the loads)
    int gl, t, gib;
    fvm::group_of<NW>(gl, t, gib);
    int L = 0;
    const bool active = colour_line(d, FAM, colour, gl, L);
    if (!active) L = 0;
    const int n = s.n;
    const LineGeo g = line_geo<FAM>(d, L);
    const double *c1, *c2, *c3, *c4;
    couple_coefs<FAM>(cf, c1, c2, c3, c4);
    T v[M];
#pragma unroll
    for (int q = 0; q < M; q++) {
        const int e = q * TG + t;
        v[q] = T(0);
        if (active && e < n) {
            const int c = g.base + e * g.stride;
            // the four transverse couplings and the source as fused multiply-adds
            v[q] = fma(lds<T>(d, c1, c), lds<T>(d, phi, c + g.o1),
                       fma(lds<T>(d, c2, c), lds<T>(d, phi, c + g.o2),
                           fma(lds<T>(d, c3, c), lds<T>(d, phi, c + g.o3),
                               fma(lds<T>(d, c4, c), lds<T>(d, phi, c + g.o4), ld<T>(SU[c])))));
        }
    }
    if (ended) return;
    fvm::to_chunks<T, M, NW>(v, sm[gib], t);
    const size_t base = size_t(L) * TG * M;
    if constexpr (std::is_same<T, double>::value) {
        fvm::group_apply<double, M, NW>(v, s.invD + base, s.fa + base, s.fb + base, t, xch[gib]);
        if (FAM != 0) fvm::group_cyclic_fix<double, M, NW>(v, s.z + base, s.cv[L], s.sinv[L], n, t, xch[gib]);
    } else {
        fvm::group_apply<dd, M, NW>(v, sd.invD + base, sd.fa + base, sd.fb + base, t, xch[gib]);
        if (FAM != 0) fvm::group_cyclic_fix<dd, M, NW>(v, sd.z + base, sd.cv[L], sd.sinv[L], n, t, xch[gib]);
    }
    fvm::to_interleaved<T, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int q = 0; q < M; q++) {
        const int e = q * TG + t;
        if (active && e < n) sts(d, phi, g.base + e * g.stride, v[q]);
    }
}

// The (hi, lo) pairs nearest to a predictor set's FP64 line factors (mixed path).
__device__ __forceinline__ dd dd_near(double x)
{
    const float h = (float)x;
    return dd(h, (float)(x - (double)h));
}
__global__ void k3_factor_dd(LineSys s, LineDD sd, size_t cnt)
{
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q < cnt) {
        sd.invD[q] = dd_near(s.invD[q]);
        sd.fa[q] = dd_near(s.fa[q]);
        sd.fb[q] = dd_near(s.fb[q]);
        if (s.cyclic) sd.z[q] = dd_near(s.z[q]);
    }
    if (s.cyclic && q < (size_t)s.lines) {
        sd.cv[q] = dd_near(s.cv[q]);
        sd.sinv[q] = dd_near(s.sinv[q]);
    }
}

}  // namespace f3

namespace f3 {

// ---------------------------------------------------------------------------------
// Explicit phase (main.f90:44-76)
// ---------------------------------------------------------------------------------
__global__ void k3_begin(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    d.U_N[c] = d.U[c];
    d.V_N[c] = d.V[c];
    d.W_N[c] = d.W[c];
    d.T_N[c] = d.T[c];
}

// CONTRA_VEL (contra_vel.f90:13-26): contravariant velocities on the whole array
__global__ void k3_contra(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const double u = d.U[c], v = d.V[c], w = d.W[c];
    d.U1[c] = (d.XIX[c] * u + d.XIY[c] * v) + d.XIZ[c] * w;
    d.U2[c] = (d.ETX[c] * u + d.ETY[c] * v) + d.ETZ[c] * w;
    d.U3[c] = (d.ZTX[c] * u + d.ZTY[c] * v) + d.ZTZ[c] * w;
}

// Face fluxes (contra_vel.f90:30-53), UW(1) = 0; with_div: the Poisson source
// DIV/dt (iter_p.f90:42-47).
__global__ void k3_fluxes(D3 d, int with_div)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const double *J = d.DJAC;
    const int c = ID3(i, j, k);
    auto f = [&](const double *Uc, int o) { return 0.5 * (J[c] * Uc[c] + J[o] * Uc[o]); };
    const double ue = f(d.U1, ID3(i + 1, j, k)), uw = (i == 1) ? 0.0 : f(d.U1, ID3(i - 1, j, k));
    const double vn = f(d.U2, ID3(i, j + 1, k)), vs = f(d.U2, ID3(i, j - 1, k));
    const double wt = f(d.U3, ID3(i, j, k + 1)), wb = f(d.U3, ID3(i, j, k - 1));
    d.UE[c] = ue; d.UW[c] = uw; d.VN[c] = vn; d.VS[c] = vs; d.WT[c] = wt; d.WB[c] = wb;
    if (with_div) d.DIVDT[c] = d.rdt * (((((ue - uw) + vn) - vs) + wt) - wb);
}

template <class T>
__device__ __forceinline__ T nl3(const D3 &d, const double *in, int c, int i, int j, int k)
{   // NL (nl.f90:23-31)
    const T p = lds<T>(d, in, c);
    return scale2(((((ld<T>(d.UE[c]) * (lds<T>(d, in, ID3(i + 1, j, k)) + p) -
                      ld<T>(d.UW[c]) * (lds<T>(d, in, ID3(i - 1, j, k)) + p)) +
                     ld<T>(d.VN[c]) * (lds<T>(d, in, ID3(i, j + 1, k)) + p)) -
                    ld<T>(d.VS[c]) * (lds<T>(d, in, ID3(i, j - 1, k)) + p)) +
                   ld<T>(d.WT[c]) * (lds<T>(d, in, ID3(i, j, k + 1)) + p)) -
                      ld<T>(d.WB[c]) * (lds<T>(d, in, ID3(i, j, k - 1)) + p),
                  0.5f);
}

// The 12 edge neighbours of a cell: (+-1,+-1,0), (+-1,0,+-1), (0,+-1,+-1) in the
// order (+,+), (+,-), (-,+), (-,-) of each pair.
__device__ __forceinline__ int edge_off(const D3 &d, int e)
{
    const int sj = d.NI1, sk = d.NI1 * d.NJ1;
    const int a = (e & 2) ? -1 : 1, b = (e & 1) ? -1 : 1;
    if (e < 4) return a + b * sj;
    if (e < 8) return a + b * sk;
    return a * sj + b * sk;
}

// A twelve-term cross derivative (dif_diagonal.f90:13-32, iter_u.f90:61-84) is
// linear in the 12 edge neighbours: with products A_xy at the cells, the
// neighbour (a, b, 0) carries 0.25 s(a) s(b) (A_12(i+a) + A_21(j+b)), and likewise
// for the (i,k) and (j,k) pairs.  The weights depend on the geometry only and are
// formed once (k3_cw); a cross term is then 12 fused multiply-adds.
template <class T = double>
__device__ __forceinline__ T cross_w(const D3 &d, double *const *W, const double *f, int c)
{
    T s = T(0);
#pragma unroll
    for (int e = 0; e < 12; e++) s = fma(lds<T>(d, W[e], c), lds<T>(d, f, c + edge_off(d, e)), s);
    return s;
}

// DIF_DIAGONAL with the J*Q weights
template <class T = double>
__device__ __forceinline__ T cross12(const D3 &d, const double *f, int i, int j, int k)
{
    return cross_w<T>(d, d.CW, f, ID3(i, j, k));
}

template <class T>
__device__ __forceinline__ T dif3(const D3 &d, const double *in, int c, int i, int j, int k)
{   // DIF (dif.f90:15-23)
    const T p = lds<T>(d, in, c);
    return (((((lds<T>(d, d.DE, c) * (lds<T>(d, in, ID3(i + 1, j, k)) - p) +
                lds<T>(d, d.DW, c) * (lds<T>(d, in, ID3(i - 1, j, k)) - p)) +
               lds<T>(d, d.DN, c) * (lds<T>(d, in, ID3(i, j + 1, k)) - p)) +
              lds<T>(d, d.DS, c) * (lds<T>(d, in, ID3(i, j - 1, k)) - p)) +
             lds<T>(d, d.DT, c) * (lds<T>(d, in, ID3(i, j, k + 1)) - p)) +
            lds<T>(d, d.DB, c) * (lds<T>(d, in, ID3(i, j, k - 1)) - p)) +
           cross12<T>(d, in, i, j, k);
}

// NL of the four fields (shifting the previous values to *_NM1), DIF of the four
// fields, P_SOURCE (p_source.f90:14-42).  T: double (FP64 path) or dd (mixed path).
template <class T>
__global__ void k3_explicit(D3 d, int thermal)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    d.NLX_NM1[c] = d.NLX[c];
    d.NLY_NM1[c] = d.NLY[c];
    d.NLZ_NM1[c] = d.NLZ[c];
    d.ADV_NM1[c] = d.ADV[c];
    d.NLX[c] = to_d(nl3<T>(d, d.U_N, c, i, j, k));
    d.NLY[c] = to_d(nl3<T>(d, d.V_N, c, i, j, k));
    d.NLZ[c] = to_d(nl3<T>(d, d.W_N, c, i, j, k));
    if (thermal) d.ADV[c] = to_d(nl3<T>(d, d.T_N, c, i, j, k));
}

// DIF of the four fields.  An FP32 sum of the FP64 inputs is no option on GB300
// (each double-to-float conversion issues on the FP64 pipe: measured 911 us against
// 625 us per launch at 256x192x48); the mixed path sums in double-float, whose loads
// split the doubles on the integer pipe.
template <class T>
__global__ void k3_dif(D3 d, int thermal)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    d.DIFX[c] = to_d(dif3<T>(d, d.U_N, c, i, j, k));
    d.DIFY[c] = to_d(dif3<T>(d, d.V_N, c, i, j, k));
    d.DIFZ[c] = to_d(dif3<T>(d, d.W_N, c, i, j, k));
    if (thermal) d.DIFT[c] = to_d(dif3<T>(d, d.T_N, c, i, j, k));
}

template <class T>
__global__ void k3_psource(D3 d)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const double *J = d.DJAC, *in = d.P;
    const int c = ID3(i, j, k), e = ID3(i + 1, j, k), w = ID3(i - 1, j, k), nn = ID3(i, j + 1, k), s = ID3(i, j - 1, k),
              t = ID3(i, j, k + 1), b = ID3(i, j, k - 1);
    const double *M1[3] = {d.XIX, d.XIY, d.XIZ}, *M2[3] = {d.ETX, d.ETY, d.ETZ}, *M3[3] = {d.ZTX, d.ZTY, d.ZTZ};
    double *out[3] = {d.S_U, d.S_V, d.S_W};
    const T Je = lds<T>(d, J, e), Jw = lds<T>(d, J, w), Jn = lds<T>(d, J, nn), Js = lds<T>(d, J, s), Jt = lds<T>(d, J, t),
            Jb = lds<T>(d, J, b);
    const T Pe = ld<T>(in[e]), Pw = ld<T>(in[w]), Pn = ld<T>(in[nn]), Ps = ld<T>(in[s]), Pt = ld<T>(in[t]),
            Pb = ld<T>(in[b]);
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const T a = (((((Je * lds<T>(d, M1[q], e)) * Pe - (Jw * lds<T>(d, M1[q], w)) * Pw) +
                       (Jn * lds<T>(d, M2[q], nn)) * Pn) -
                      (Js * lds<T>(d, M2[q], s)) * Ps) +
                     (Jt * lds<T>(d, M3[q], t)) * Pt) -
                    (Jb * lds<T>(d, M3[q], b)) * Pb;
        out[q][c] = to_d(scale2(a, -0.5f));
    }
}

// Far-field values of BCU/BCT (bcu.f90:30-40) from the step-n fields, per (j,k):
// inflow value where THETA(NI) in [pi/2, 3pi/2], else the convective outflow value.
__global__ void k3_farfield(D3 d)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (j > d.NJ - 1 || k > d.NK - 1) return;
    const int i = d.NI;
    const double th = d.THETA[ID3(i, j, k)];
    const bool inflow = th >= 0.5 * d.pi && th <= 1.5 * d.pi;
    const double *B[4] = {d.U_N, d.V_N, d.W_N, d.T_N};
    double *out[4] = {d.FFU, d.FFV, d.FFW, d.FFT};
    const double fin[4] = {1.0, 0.0, 0.0, d.tin};
    const double a = 0.5 * (d.XIX[ID3(i, j, k)] + d.XIX[ID3(i - 1, j, k)]);
    const double b = (0.5 * (d.ETX[ID3(i, j, k)] + d.ETX[ID3(i - 1, j, k)])) * 0.25;
    const double cz = (0.5 * (d.ZTX[ID3(i, j, k)] + d.ZTX[ID3(i - 1, j, k)])) * 0.25;
    for (int q = 0; q < 4; q++) {
        const double *q3 = B[q];
        double f = fin[q];
        if (!inflow)
            f = 0.5 * (q3[ID3(i, j, k)] + q3[ID3(i - 1, j, k)]) -
                (d.dt * 1.0) *
                    ((a * (q3[ID3(i, j, k)] - q3[ID3(i - 1, j, k)]) +
                      b * (((q3[ID3(i, j + 1, k)] + q3[ID3(i - 1, j + 1, k)]) - q3[ID3(i, j - 1, k)]) - q3[ID3(i - 1, j - 1, k)])) +
                     cz * (((q3[ID3(i, j, k + 1)] + q3[ID3(i - 1, j, k + 1)]) - q3[ID3(i, j, k - 1)]) - q3[ID3(i - 1, j, k - 1)]));
        out[q][JK(j, k)] = f;
    }
}

// BCU/BCT (bcu.f90:26, 45): the wall ghost from the first cell of every (j,k) line,
// the far-field ghost from the last cell and the far-field value (kind 2 is the
// temperature, wall value T_WALL), followed by the periodic copy of the field, in one
// launch: every ghost gets the value that sequence produces, from interior values only --
// the wall ghost -phi(1) + 2 u_w and the far-field ghost -phi(NI-1) + 2 ff of the
// wrapped (j, k), and phi(i, wrapped j, wrapped k) on the J and K ghost planes.
// Threads [0, nin): the two I ghosts of the interior line (j, k); the others: cell i
// of a ghost row (j in {0, NJ} or k in {0, NK}; the K-plane rows first).  Mixed
// path: the ghosts' shadows too.
__global__ void k3_bcu(D3 d, double *phi, const double *ff, int kind)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int nj1 = d.NJ - 1, nk1 = d.NK - 1;
    const long long nin = (long long)nj1 * nk1;
    const long long nrow = 2LL * (d.NJ + 1) + 2LL * nk1;
    if (t >= nin + nrow * d.NI1) return;
    const double uf = kind == 2 ? d.t_wall : 0.0;
    auto put = [&](int c, double v) {
        phi[c] = v;
        if (d.dfl) {
            const dd s = fvm::dd_split(v);
            shadow(d, phi)[c] = make_float2(s.hi, s.lo);
        }
    };
    int i, j, k;
    if (t < nin) {
        j = (int)(t % nj1) + 1;
        k = (int)(t / nj1) + 1;
        put(ID3(0, j, k), (-phi[ID3(1, j, k)]) + 2.0 * uf);
        put(ID3(d.NI, j, k), (-phi[ID3(d.NI - 1, j, k)]) + 2.0 * ff[JK(j, k)]);
        return;
    }
    const long long q = t - nin;
    const int r = (int)(q / d.NI1);
    i = (int)(q % d.NI1);
    if (r < 2 * (d.NJ + 1)) {   // K ghost planes, every j
        k = r < d.NJ + 1 ? 0 : d.NK;
        j = r % (d.NJ + 1);
    } else {                    // J ghost planes, interior k
        const int r2 = r - 2 * (d.NJ + 1);
        j = r2 < nk1 ? 0 : d.NJ;
        k = r2 % nk1 + 1;
    }
    const int js = jw(d, j), ks = kw(d, k), c = ID3(i, j, k);
    if (i == 0) put(c, (-phi[ID3(1, js, ks)]) + 2.0 * uf);
    else if (i == d.NI) put(c, (-phi[ID3(d.NI - 1, js, ks)]) + 2.0 * ff[JK(js, ks)]);
    else put(c, phi[ID3(i, js, ks)]);
}

// Right-hand side of one AF sweep (iter_u.f90:44-100, iter_T.f90): the split's
// twelve cross terms of phi, the sweep's source, and the BC folding of BCU/BCT.
// T: double (FP64 path) or dd (mixed path, where 2 Re J / dt is J times the
// precomputed 2 Re / dt instead of a division per cell).
template <class T>
__global__ void k3_af_rhs(D3 d, Coef3 cf, int split, int kind, const double *phi, const double *phin,
                          const double *ina, const double *inb, const double *inc, const double *ind,
                          const double *ff)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    const double *J = d.DJAC;
    const T cr = cross_w<T>(d, d.CWA[split], phi, c);
    const double rek = kind == 2 ? d.pe : d.re;
    T r;
    if constexpr (std::is_same<T, double>::value) r = ((2.0 * rek) * J[c]) / d.dt;
    else r = lds<T>(d, J, c) * ld<T>(kind == 2 ? d.r2pe_dt : d.r2re_dt);
    T su;
    if (split == 0) {
        const T re1 = ld<T>(rek);
        su = (r * lds<T>(d, phin, c) - (T(3) * re1) * ld<T>(ina[c])) + re1 * ld<T>(inb[c]);
        su = su + ld<T>(inc[c]);
        if (ind) su = su + scale2(re1, 2.0f) * ld<T>(ind[c]);
        su = su + cr;
    } else {
        su = r * lds<T>(d, phi, c) + cr;
    }
    const double uf = kind == 2 ? d.t_wall : 0.0;
    if (i == 1) su = su + scale2(ld<T>(cf.awall[JK(j, k)]), 2.0f) * ld<T>(uf);
    if (i == d.NI - 1) su = su + scale2(ld<T>(cf.afar[JK(j, k)]), 2.0f) * ld<T>(ff[JK(j, k)]);
    d.SU[c] = to_d(su);
}

// u += sign * dt * S / J (main.f90:84-86, 104-106).  The update of the state is
// FP64 in both paths; the mixed path forms the increments dt S / J in double-float.
template <class T>
__global__ void k3_grad(D3 d, double sign)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    if constexpr (!std::is_same<T, double>::value) {
        const T rj = T(1) / lds<T>(d, d.DJAC, c), f = ld<T>(d.dt);
        const double iu = to_d((f * ld<T>(d.S_U[c])) * rj), iv = to_d((f * ld<T>(d.S_V[c])) * rj),
                     iw = to_d((f * ld<T>(d.S_W[c])) * rj);
        if (sign < 0) {
            d.U[c] = d.U[c] - iu;
            d.V[c] = d.V[c] - iv;
            d.W[c] = d.W[c] - iw;
        } else {
            d.U[c] = d.U[c] + iu;
            d.V[c] = d.V[c] + iv;
            d.W[c] = d.W[c] + iw;
        }
        return;
    }
    const double f = d.dt;
    if (sign < 0) {
        d.U[c] = d.U[c] - (f * d.S_U[c]) / d.DJAC[c];
        d.V[c] = d.V[c] - (f * d.S_V[c]) / d.DJAC[c];
        d.W[c] = d.W[c] - (f * d.S_W[c]) / d.DJAC[c];
    } else {
        d.U[c] = d.U[c] + (f * d.S_U[c]) / d.DJAC[c];
        d.V[c] = d.V[c] + (f * d.S_V[c]) / d.DJAC[c];
        d.W[c] = d.W[c] + (f * d.S_W[c]) / d.DJAC[c];
    }
}

// ---------------------------------------------------------------------------------
// ITER_P (iter_p.f90:37-63): source with the lagged cross term, BCP ghosts,
// red-black I-line sweep, scaled residual
// ---------------------------------------------------------------------------------
__global__ void k3_psu(D3 d)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    if (d.pctl->done) return;
    d.SU[c] = d.DIVDT[c] - cross12(d, d.P, i, j, k);
}

// BCP ghosts (bcp.f90:24-34): P(0) = P(1), P(NI) cubic extrapolation (periodic
// copy follows).  check_done: part of the Poisson loop.
__global__ void k3_bcp(D3 d, int check_done)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y;
    if (j > d.NJ - 1 || k > d.NK) return;
    if (check_done && d.pctl->done) return;
    double *P = d.P;
    P[ID3(0, j, k)] = P[ID3(1, j, k)];
    P[ID3(d.NI, j, k)] = (3.0 * P[ID3(d.NI - 1, j, k)] - 3.0 * P[ID3(d.NI - 2, j, k)]) + P[ID3(d.NI - 3, j, k)];
}

// Block sum of three values (warp shuffle trees, then the warps in order; thread 0
// holds the result).
__device__ __forceinline__ void block_sum3(double &a, double &b, double &e, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        e += __shfl_down_sync(0xffffffffu, e, o);
    }
    const int wid = threadIdx.x / WARP, lane = threadIdx.x & 31, nw = blockDim.x / WARP;
    __syncthreads();   // sh may hold an earlier round's values
    if (lane == 0) { sh[3 * wid] = a; sh[3 * wid + 1] = b; sh[3 * wid + 2] = e; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0, z = 0.0;
        for (int w = 0; w < nw; w++) { x += sh[3 * w]; y += sh[3 * w + 1]; z += sh[3 * w + 2]; }
        a = x;
        b = y;
        e = z;
    }
}

// Deterministic two-level sum of three values over the grid: each block's sum goes
// to `partial`; the last block to arrive sums the partials with all its threads
// (a fixed strided assignment, then the block tree).  Returns true in the last
// block, whose thread 0 holds the sums.
__device__ bool grid_sum3(const D3 &d, double &a, double &b, double &e, double *sh, bool &last, unsigned *ticket)
{
    block_sum3(a, b, e, sh);
    if (threadIdx.x == 0) {
        d.partial[4 * blockIdx.x] = a;
        d.partial[4 * blockIdx.x + 1] = b;
        d.partial[4 * blockIdx.x + 2] = e;
        __threadfence();
        unsigned t = atomicInc(ticket, gridDim.x - 1);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    a = 0.0;
    b = 0.0;
    e = 0.0;
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) {
        a += ((volatile double *)d.partial)[4 * q];
        b += ((volatile double *)d.partial)[4 * q + 1];
        e += ((volatile double *)d.partial)[4 * q + 2];
    }
    block_sum3(a, b, e, sh);
    return true;
}

// HAS_COND: the device-loop form, which ends the graph while node; a separate
// instantiation keeps the host-loop kernels free of device graph calls (profilers
// skip kernels that contain them).
template <int HAS_COND>
__global__ void __launch_bounds__(256) k3_pres(D3 d, Coef3 cf, int per, cudaGraphConditionalHandle cond)
{
    __shared__ double sh[3 * 8];
    __shared__ bool last;
    if (d.pctl->done) return;
    const int ni1 = d.NI - 1, nj1 = d.NJ - 1, total = ni1 * nj1 * (d.NK - 1);
    double ra = 0.0, pa = 0.0, dummy = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int i = e % ni1 + 1, j = (e / ni1) % nj1 + 1, k = e / (ni1 * nj1) + 1, c = ID3(i, j, k);
        const double *P = d.P;
        double r = ((((((cf.AE[c] * P[ID3(i + 1, j, k)] + cf.AW[c] * P[ID3(i - 1, j, k)]) +
                        cf.AN[c] * P[ID3(i, jw(d, j + 1), k)]) + cf.AS[c] * P[ID3(i, jw(d, j - 1), k)]) +
                      cf.AT[c] * P[ID3(i, j, kw(d, k + 1))]) + cf.AB[c] * P[ID3(i, j, kw(d, k - 1))]) +
                    d.SU[c]) - cf.AP[c] * P[c];
        ra += fabs(r);
        pa += fabs(cf.AP[c] * P[c]);
    }
    if (!grid_sum3(d, ra, pa, dummy, sh, last, &d.pctl->ticket)) return;
    if (threadIdx.x == 0) {
        const int it = d.pctl->niter + per;
        const double resip = ra / pa;
        d.pctl->niter = it;
        d.pctl->resip = resip;
        if (!(resip > d.resimax && it < d.nswpp)) {
            d.pctl->done = 1;
            d.pctl->capped = resip > d.resimax ? 1 : 0;
            if constexpr (HAS_COND) cudaGraphSetConditional(cond, 0);   // ends the device-side loop
        }
    }
}

__global__ void k3_pctl_reset(D3 d)
{
    d.pctl->niter = 0;
    d.pctl->done = 0;
    d.pctl->capped = 0;
    d.pctl->resip = 0.0;
}

// Reference pressure (main.f90:125-135): the span average of P(NI, NJ/4, k)
// subtracted from the whole array (one block computes the average first).
__global__ void k3_pref(D3 d)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int k = 1; k <= d.NK - 1; k++) s = s + d.P[ID3(d.NI, d.NJ / 4, k)];
    d.scal[2] = s / (double)(d.NK - 1);
}

__global__ void k3_pshift(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    d.P[c] = d.P[c] - d.scal[2];
}

// ---------------------------------------------------------------------------------
// MIXED Poisson: FP64 defect correction around FP32 red-black I-line sweeps.  Each
// outer iteration forms in FP64 the full residual r = SU - A P, with the cross
// term of SU recomputed from the current P (iter_p.f90:37-63, dif_diagonal.f90:
// 13-32), its scaled-L1 norm (the convergence test of iter_p.f90:43-63) and r in
// FP32; refine_sweeps FP32 sweeps then solve A7 dP = r from dP = 0 with the FP32
// line factors, and P += dP in FP64 with the BCP ghosts and the periodic copy
// refreshed.  The fixed point is the one of the FP64 iteration.
// ---------------------------------------------------------------------------------
__global__ void k3_coef_f32(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const Coef3 &cf = d.cf[6];
    d.ANf[c] = (float)cf.AN[c];
    d.ATf[c] = (float)cf.AT[c];
}

template <int HAS_COND>
__global__ void __launch_bounds__(256) k3_mres(D3 d, cudaGraphConditionalHandle cond)
{
    __shared__ double sh[3 * 8];
    __shared__ bool last;
    if (d.pctl->done) return;
    const int it = d.pctl->niter;
    const Coef3 &cf = d.cf[6];
    const int ni1 = d.NI - 1, nj1 = d.NJ - 1, total = ni1 * nj1 * (d.NK - 1);
    double ra = 0.0, pa = 0.0, dummy = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int i = e % ni1 + 1, j = (e / ni1) % nj1 + 1, k = e / (ni1 * nj1) + 1, c = ID3(i, j, k);
        const double *P = d.P;
        const double su = d.DIVDT[c] - cross12(d, P, i, j, k);
        const double r = ((((((cf.AE[c] * P[ID3(i + 1, j, k)] + cf.AW[c] * P[ID3(i - 1, j, k)]) +
                              cf.AN[c] * P[ID3(i, jw(d, j + 1), k)]) + cf.AS[c] * P[ID3(i, jw(d, j - 1), k)]) +
                            cf.AT[c] * P[ID3(i, j, kw(d, k + 1))]) + cf.AB[c] * P[ID3(i, j, kw(d, k - 1))]) + su) -
                         cf.AP[c] * P[c];
        ra += fabs(r);
        pa += fabs(cf.AP[c] * P[c]);
        d.RF[c] = (float)r;
        d.DF[c] = 0.0f;
    }
    if (!grid_sum3(d, ra, pa, dummy, sh, last, &d.pctl->ticket)) return;
    if (threadIdx.x == 0) {
        const double resip = ra / pa;
        d.pctl->resip = resip;
        if (it > 0 && !(resip > d.resimax && it < d.nswpp)) {
            d.pctl->done = 1;
            d.pctl->capped = resip > d.resimax ? 1 : 0;
            if constexpr (HAS_COND) cudaGraphSetConditional(cond, 0);   // ends the device-side loop
        } else {
            d.pctl->niter = it + d.refine_sweeps;
        }
    }
}

// BCP ghosts of the I line (j, k) of P (bcp.f90:24-34): P(0) = P(1), P(NI) cubic.
__device__ __forceinline__ void line_bcp(const D3 &d, int j, int k)
{
    double *P = d.P;
    P[ID3(0, j, k)] = P[ID3(1, j, k)];
    P[ID3(d.NI, j, k)] = (3.0 * P[ID3(d.NI - 1, j, k)] - 3.0 * P[ID3(d.NI - 2, j, k)]) + P[ID3(d.NI - 3, j, k)];
}

// One colour of the FP32 correction sweep on the I lines of the Poisson set.  The
// south and bottom couplings are the north and top couplings of the neighbouring
// lines.  apply != 0 (the colour-1 launch of the last sweep of an outer iteration):
// the group also adds the correction to P on its own line and on its colour-0
// partner line (j-1, k) -- j -> j-1 maps the colour-1 lines of a plane one to one
// onto the colour-0 lines -- and sets the BCP ghosts of both lines.
template <int M, int NW>
__global__ void __launch_bounds__(128) k3_line32(D3 d, LineSys s, int colour, int check_done, int apply)
{
    constexpr int TG = WARP * NW, G = 4 / NW;
    __shared__ float sm[G][TG * M + M * NW + 1];
    __shared__ float xch[G][2 * NW];
    // the loop's done flag is loaded together with the operands below
    const int stop = check_done ? d.pctl->done : 0;
    int gl, t, gib;
    fvm::group_of<NW>(gl, t, gib);
    int L = 0;
    const bool active = colour_line(d, 0, colour, gl, L);
    if (!active) L = 0;
    const int n = s.n, j = L % (d.NJ - 1) + 1, k = L / (d.NJ - 1) + 1;
    const int jn = jw(d, j + 1), js = jw(d, j - 1), kt = kw(d, k + 1), kb = kw(d, k - 1);
    const float *DF = d.DF;
    float v[M];
#pragma unroll
    for (int q = 0; q < M; q++) {
        const int e = q * TG + t;
        v[q] = 0.0f;
        if (active && e < n) {
            const int i = e + 1, c = ID3(i, j, k);
            v[q] = ((d.ANf[c] * DF[ID3(i, jn, k)] + d.ANf[ID3(i, js, k)] * DF[ID3(i, js, k)]) +
                    (d.ATf[c] * DF[ID3(i, j, kt)] + d.ATf[ID3(i, j, kb)] * DF[ID3(i, j, kb)])) + d.RF[c];
        }
    }
    if (stop) return;
    fvm::to_chunks<float, M, NW>(v, sm[gib], t);
    const size_t base = size_t(L) * TG * M;
    fvm::group_apply<float, M, NW>(v, s.invDf + base, s.faf + base, s.fbf + base, t, xch[gib]);
    fvm::to_interleaved<float, M, NW>(v, sm[gib], t);
#pragma unroll
    for (int q = 0; q < M; q++) {
        const int e = q * TG + t;
        if (active && e < n) d.DF[ID3(e + 1, j, k)] = v[q];
    }
    if (!apply) return;
#pragma unroll
    for (int q = 0; q < M; q++) {
        const int e = q * TG + t;
        if (active && e < n) {
            d.P[ID3(e + 1, j, k)] += fvm::f2d_int(v[q]);
            d.P[ID3(e + 1, js, k)] += fvm::f2d_int(DF[ID3(e + 1, js, k)]);
        }
    }
    fvm::gsync<NW>();
    if (active && t == 0) {
        __threadfence_block();
        line_bcp(d, j, k);
        line_bcp(d, js, k);
    }
}


}  // namespace f3

namespace f3 {

// ---------------------------------------------------------------------------------
// Dynamic Smagorinsky model (stress_tensor_dy.f90:20-735, test_filter.f90:13-21)
// ---------------------------------------------------------------------------------
// The model's stencils are templates over the arithmetic type T and are instantiated
// with double in both precision modes: the Leonard term filt(u_i u_j) - û_i û_j is
// a difference of O(1) numbers that is ~1e-6 on a wall-resolved grid, so FP32
// arithmetic leaves it with ~10 % error.
template <class T>
__device__ __forceinline__ T dxi(const D3 &d, const double *m, const double *f, int i, int j, int k)
{
    const int c = ID3(i, j, k);
    if (i == 0) return scale2(lds<T>(d, m, c), 2.0f) * (lds<T>(d, f, ID3(1, j, k)) - lds<T>(d, f, c));
    if (i == d.NI) return scale2(lds<T>(d, m, c), 2.0f) * (lds<T>(d, f, c) - lds<T>(d, f, ID3(d.NI - 1, j, k)));
    return lds<T>(d, m, c) * (lds<T>(d, f, ID3(i + 1, j, k)) - lds<T>(d, f, ID3(i - 1, j, k)));
}
template <class T>
__device__ __forceinline__ T deta(const D3 &d, const double *m, const double *f, int i, int j, int k)
{
    return lds<T>(d, m, ID3(i, j, k)) * (lds<T>(d, f, ID3(i, j + 1, k)) - lds<T>(d, f, ID3(i, j - 1, k)));
}
template <class T>
__device__ __forceinline__ T dzeta(const D3 &d, const double *m, const double *f, int i, int j, int k)
{
    return lds<T>(d, m, ID3(i, j, k)) * (lds<T>(d, f, ID3(i, j, k + 1)) - lds<T>(d, f, ID3(i, j, k - 1)));
}

// Strain-rate components S11..S33 of (u,v,w) (0.5 / 0.25 times the index-difference
// sums) and, with t, the temperature gradient (0.5 times the sums).
template <class T>
__device__ void strain3(const D3 &d, const double *u, const double *v, const double *w, const double *t, int i, int j,
                        int k, T *S, T *G)
{
    const double *M1[3] = {d.XIX, d.XIY, d.XIZ}, *M2[3] = {d.ETX, d.ETY, d.ETZ}, *M3[3] = {d.ZTX, d.ZTY, d.ZTZ};
    const double *F[3] = {u, v, w};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = a; b < 3; b++) {
            T val;
            if (a == b) {
                val = scale2((dxi<T>(d, M1[a], F[a], i, j, k) + deta<T>(d, M2[a], F[a], i, j, k)) +
                                 dzeta<T>(d, M3[a], F[a], i, j, k),
                             0.5f);
            } else {
                T s = dxi<T>(d, M1[b], F[a], i, j, k);
                s = s + deta<T>(d, M2[b], F[a], i, j, k);
                s = s + dzeta<T>(d, M3[b], F[a], i, j, k);
                s = s + dxi<T>(d, M1[a], F[b], i, j, k);
                s = s + deta<T>(d, M2[a], F[b], i, j, k);
                s = s + dzeta<T>(d, M3[a], F[b], i, j, k);
                val = scale2(s, 0.25f);
            }
            S[3 * a + b] = val;
            S[3 * b + a] = val;
        }
    if (t)
#pragma unroll
        for (int q = 0; q < 3; q++)
            G[q] = scale2((dxi<T>(d, M1[q], t, i, j, k) + deta<T>(d, M2[q], t, i, j, k)) + dzeta<T>(d, M3[q], t, i, j, k),
                          0.5f);
}

template <class T>
__device__ __forceinline__ T sq9(const T *S)
{
    T s = S[0] * S[0];
#pragma unroll
    for (int q = 1; q < 9; q++) s = s + S[q] * S[q];
    return s;
}

// 6 blocks of 128 threads per SM (80 registers, no spills): 24 warps instead of 16
template <class T>
__global__ void __launch_bounds__(128, 6) k3_strain(D3 d)
{
    CELL3(0, d.NI, 1, d.NJ - 1, 1, d.NK - 1)
    T S[9], G[3];
    strain3<T>(d, d.U, d.V, d.W, d.T, i, j, k, S, G);
    const int c = ID3(i, j, k);
#pragma unroll
    for (int q = 0; q < 9; q++) sts(d, d.L[q], c, S[q]);
#pragma unroll
    for (int q = 0; q < 3; q++) sts(d, d.DTD[q], c, G[q]);
}

template <class T>
__global__ void k3_mag(D3 d)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    T s = lds<T>(d, d.L[0], c) * lds<T>(d, d.L[0], c);
#pragma unroll
    for (int q = 1; q < 9; q++) s = s + lds<T>(d, d.L[q], c) * lds<T>(d, d.L[q], c);
    sts(d, d.MAG, c, sqrt(scale2(s, 2.0f)));
}

// [1,2,1]^3 / 64 over the 27 neighbours of an interior cell, the reference's term
// order (K-1 plane first, I fastest).
template <class T>
__device__ __forceinline__ T filt(const D3 &d, const double *in, int i, int j, int k)
{
    T s = T(0);
    bool first = true;
#pragma unroll
    for (int c = -1; c <= 1; c++)
#pragma unroll
        for (int b = -1; b <= 1; b++)
#pragma unroll
            for (int a = -1; a <= 1; a++) {
                const T wt = T((2 - (a * a)) * (2 - (b * b)) * (2 - (c * c)));
                const T v = T(in[ID3(i + a, j + b, k + c)]);
                const T term = wt == T(1) ? v : wt * v;
                s = first ? term : s + term;
                first = false;
            }
    return s / T(64);
}

template <class T>
__global__ void k3_filter(D3 d, const double *in, double *out)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    out[ID3(i, j, k)] = (double)filt<T>(d, in, i, j, k);
}

// ---------------------------------------------------------------------------------
// The test filter (test_filter.f90:13-21) applied separably: the [1,2,1]^3/64 box
// filter is the product of three [1,2,1] passes, I, J, then K with the 1/64, so
// the 22 filters of a step (the filtered velocity and temperature, the Germano
// products, the heat-flux products) read each input three times instead of 27.
// Bank b, array q at FB + (12 b + q) n.  The result is the reference's 27-point
// sum up to rounding (the terms are added in another order).
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double *fbank(const D3 &d, int b, int q) { return d.FB + (size_t(12 * b + q)) * d.n; }
// Bank elements hold doubles in the FP64 path and (hi, lo) pairs in the mixed path.
template <class T>
__device__ __forceinline__ T bank_ld(const D3 &d, int b, int q, int c);
template <>
__device__ __forceinline__ double bank_ld<double>(const D3 &d, int b, int q, int c) { return fbank(d, b, q)[c]; }
template <>
__device__ __forceinline__ dd bank_ld<dd>(const D3 &d, int b, int q, int c)
{
    const float2 v = reinterpret_cast<const float2 *>(fbank(d, b, q))[c];
    return dd(v.x, v.y);
}
__device__ __forceinline__ void bank_st(const D3 &d, int b, int q, int c, double v) { fbank(d, b, q)[c] = v; }
__device__ __forceinline__ void bank_st(const D3 &d, int b, int q, int c, dd v)
{
    reinterpret_cast<float2 *>(fbank(d, b, q))[c] = make_float2(v.hi, v.lo);
}

enum { SEP_HATS = 0, SEP_VEL = 1, SEP_HEAT = 2 };

// Filter inputs over the whole array into bank 0: U, V, W, T (SEP_HATS); the
// velocity products uu, vv, ww, uv, uw, vw and MAG*S11, S22, S33, S12, S13, S23
// (SEP_VEL, stress_tensor_dy.f90:266-483); uT, vT, wT and MAG*dT/dx_q (SEP_HEAT,
// stress_tensor_dy.f90:590-680).
template <class T>
__global__ void k3_prod(D3 d, int mode)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const T u = lds<T>(d, d.U, c), v = lds<T>(d, d.V, c), w = lds<T>(d, d.W, c), t = lds<T>(d, d.T, c);
    if (mode == SEP_HATS) {
        bank_st(d, 0, 0, c, u);
        bank_st(d, 0, 1, c, v);
        bank_st(d, 0, 2, c, w);
        bank_st(d, 0, 3, c, t);
    } else if (mode == SEP_VEL) {
        const T mg = lds<T>(d, d.MAG, c);
        const T uv[3] = {u, v, w};
#pragma unroll
        for (int q = 0; q < 6; q++) {
            const int a = q < 3 ? q : (q == 5 ? 1 : 0), b = q < 3 ? q : (q == 3 ? 1 : 2);
            bank_st(d, 0, q, c, uv[a] * uv[b]);
            bank_st(d, 0, 6 + q, c, mg * lds<T>(d, d.L[3 * a + b], c));
        }
    } else {
        const T mg = lds<T>(d, d.MAG, c);
        bank_st(d, 0, 0, c, u * t);
        bank_st(d, 0, 1, c, v * t);
        bank_st(d, 0, 2, c, w * t);
#pragma unroll
        for (int q = 0; q < 3; q++) bank_st(d, 0, 3 + q, c, mg * lds<T>(d, d.DTD[q], c));
    }
}

struct Out4 {
    double *p[4];
};

// One [1,2,1] pass over nq arrays from bank src to bank dst: dir 0 (I) for
// i = 1..NI-1 on every (j, k); dir 1 (J) for j = 1..NJ-1 on every k; dir 2 (K) on
// the interior, with the 1/64, into bank dst or, when out.p[0] is set, into out.p[q].
template <class T>
__global__ void k3_sep(D3 d, int src, int dst, int nq, int dir, Out4 out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + (dir == 0 ? 0 : 1);
    const int k = blockIdx.z + (dir == 2 ? 1 : 0);
    if (i > d.NI - 1 || j > (dir == 0 ? d.NJ : d.NJ - 1) || k > (dir == 2 ? d.NK - 1 : d.NK)) return;
    const int c = ID3(i, j, k), o = dir == 0 ? 1 : (dir == 1 ? d.NI1 : d.NI1 * d.NJ1);
    for (int q = 0; q < nq; q++) {
        const T r = (bank_ld<T>(d, src, q, c - o) + scale2(bank_ld<T>(d, src, q, c), 2.0f)) + bank_ld<T>(d, src, q, c + o);
        if (dir != 2) bank_st(d, dst, q, c, r);
        else if (out.p[0]) out.p[q][c] = to_d(scale2(r, 1.0f / 64.0f));
        else bank_st(d, dst, q, c, scale2(r, 1.0f / 64.0f));
    }
}

// Germano terms of the six velocity components (11, 22, 33, 12, 13, 23) from the
// filtered products in bank b, accumulated into LM and MM in that order with the
// off-diagonal ones weighted 2; the strain rate of the filtered velocity and its
// magnitude once per cell (MAGH is kept for the heat flux).
template <class T>
__global__ void __launch_bounds__(128, 6) k3_germano(D3 d, int b)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    const double *uh[3] = {d.UH, d.VH, d.WH};
    T S[9], G[3];
    strain3<T>(d, d.UH, d.VH, d.WH, nullptr, i, j, k, S, G);
    const T magh = sqrt(scale2(sq9<T>(S), 2.0f));
    d.MAGH[c] = to_d(magh);
    const T fw2 = lds<T>(d, d.FW, c) * lds<T>(d, d.FW, c);
    T lm, mm;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const int a = q < 3 ? q : (q == 5 ? 1 : 0), bb = q < 3 ? q : (q == 3 ? 1 : 2);
        const T l = (-bank_ld<T>(d, b, q, c)) + lds<T>(d, uh[a], c) * lds<T>(d, uh[bb], c);
        const T dout = bank_ld<T>(d, b, 6 + q, c);
        // fac = 0.5 on the diagonal, 0.25 off it: hs = S / fac, m = ((4 magh) fac) hs
        const float fac = a == bb ? 0.5f : 0.25f;
        const T hs = scale2(S[3 * a + bb], 1.0f / fac);
        T m = scale2(scale2(magh, 4.0f), fac) * hs;
        m = fw2 * (m - dout);
        if (q == 0) {
            lm = l * m;
            mm = m * m;
        } else if (q < 3) {
            lm = lm + l * m;
            mm = mm + m * m;
        } else {
            lm = lm + scale2(l, 2.0f) * m;
            mm = mm + scale2(m, 2.0f) * m;
        }
    }
    d.LM[c] = to_d(lm);
    d.MM[c] = to_d(mm);
}

// Temperature terms P_q, R_q of the three heat-flux components from the filtered
// products in bank b, accumulated into LM and MM.
template <class T>
__global__ void k3_germano_t(D3 d, int b)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    const double *uh[3] = {d.UH, d.VH, d.WH};
    const double *M1[3] = {d.XIX, d.XIY, d.XIZ}, *M2[3] = {d.ETX, d.ETY, d.ETZ}, *M3[3] = {d.ZTX, d.ZTY, d.ZTZ};
    const T fw2 = lds<T>(d, d.FW, c) * lds<T>(d, d.FW, c), magh = ld<T>(d.MAGH[c]);
    T lm, mm;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const T l = (-bank_ld<T>(d, b, q, c)) + lds<T>(d, uh[q], c) * lds<T>(d, d.TH, c);
        const T dout = bank_ld<T>(d, b, 3 + q, c);
        const T g = (dxi<T>(d, M1[q], d.TH, i, j, k) + deta<T>(d, M2[q], d.TH, i, j, k)) +
                    dzeta<T>(d, M3[q], d.TH, i, j, k);
        T m = scale2(scale2(magh, 4.0f), 0.5f) * g;
        m = fw2 * (m - dout);
        if (q == 0) {
            lm = l * m;
            mm = m * m;
        } else {
            lm = lm + l * m;
            mm = mm + m * m;
        }
    }
    d.LM[c] = to_d(lm);
    d.MM[c] = to_d(mm);
}

// (0.5 lm) / mm >= 0, decided without the division (one FP64 division costs several
// FP64-pipe instructions on GB300) and exactly as the quotient would decide it,
// including zero, infinite and NaN operands and a negative quotient that underflows
// to -0 (|q| <= 2^-1075).
__device__ __forceinline__ bool coef_nonneg(double lm, double mm)
{
    const double h = 0.5 * lm;
    if (h != h || mm != mm) return false;
    const double ah = fabs(h), am = fabs(mm);
    const bool same = signbit(h) == signbit(mm);
    if (am == 0.0) return h != 0.0 && same;                     // +-inf or NaN
    if (am > DBL_MAX) return ah <= DBL_MAX;                     // finite / inf = +-0
    if (ah > DBL_MAX) return same;                              // inf / finite
    if (same) return true;                                      // positive or +-0
    return (ah * 0x1p600) * 0x1p475 <= am;                      // rounds to -0
}

// Volume-averaged coefficient over the points whose local coefficient is >= 0
// (stress_tensor_dy.f90:486-517): result in scal[slot].
__global__ void __launch_bounds__(256) k3_cvol(D3 d, int slot)
{
    __shared__ double sh[3 * 8];
    __shared__ bool last;
    const int ni1 = d.NI - 1, nj1 = d.NJ - 1, total = ni1 * nj1 * (d.NK - 1);
    double lm = 0.0, mm = 0.0, inc = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int i = e % ni1 + 1, j = (e / ni1) % nj1 + 1, k = e / (ni1 * nj1) + 1, c = ID3(i, j, k);
        if (coef_nonneg(d.LM[c], d.MM[c])) {
            lm += d.LM[c];
            mm += d.MM[c];
            inc += 1.0;
        }
    }
    if (!grid_sum3(d, lm, mm, inc, sh, last, &d.pctl->ticket)) return;
    if (threadIdx.x == 0) {
        lm = lm / inc;
        mm = mm / inc;
        double cavg = (0.5 * lm) / mm;
        if (mm < 1e-6) cavg = 0.0;
        d.scal[slot] = cavg;
    }
}

// Lilly least squares along the span per (i,j), clipped at zero.
__global__ void k3_czavg(D3 d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
    if (i > d.NI - 1 || j > d.NJ - 1) return;
    double lm = 0.0, mm = 0.0;
    for (int k = 1; k <= d.NK - 1; k++) {
        lm = lm + d.LM[ID3(i, j, k)];
        mm = mm + d.MM[ID3(i, j, k)];
    }
    const double cc = mm > 0.0 ? (0.5 * lm) / mm : 0.0;
    d.CZ[i + d.NI1 * j] = cc > 0.0 ? cc : 0.0;
}

__global__ void k3_eddy(D3 d, int slot, double *out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    double cc = d.scal[slot];
    if (d.les_zavg) {
        const int i = c % d.NI1, j = (c / d.NI1) % d.NJ1;
        const int ii = i < 1 ? 1 : (i > d.NI - 1 ? d.NI - 1 : i);
        cc = d.CZ[ii + d.NI1 * jw(d, j)];
    }
    out[c] = (cc * (d.FW[c] * d.FW[c])) * d.MAG[c];
    if (d.dfl) {
        const dd v = fvm::dd_split(out[c]);
        shadow(d, out)[c] = make_float2(v.hi, v.lo);
    }
}

template <class T>
__device__ __forceinline__ T sgs_div(const D3 &d, const double *E, const double *const *Lc, int i, int j, int k)
{
    const double *M1[3] = {d.XIX, d.XIY, d.XIZ}, *M2[3] = {d.ETX, d.ETY, d.ETZ}, *M3[3] = {d.ZTX, d.ZTY, d.ZTZ};
    const int c = ID3(i, j, k), ip = ID3(i + 1, j, k), im = ID3(i - 1, j, k), jp = ID3(i, j + 1, k),
              jm = ID3(i, j - 1, k), kp = ID3(i, j, k + 1), km = ID3(i, j, k - 1);
    // 2 E at the six neighbours
    const T ep = scale2(lds<T>(d, E, ip), 2.0f), em = scale2(lds<T>(d, E, im), 2.0f),
            fp = scale2(lds<T>(d, E, jp), 2.0f), fm = scale2(lds<T>(d, E, jm), 2.0f),
            gp = scale2(lds<T>(d, E, kp), 2.0f), gm = scale2(lds<T>(d, E, km), 2.0f);
    T s;
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const double *L = Lc[b];
        const T t1 = lds<T>(d, M1[b], c) * (-(ep * lds<T>(d, L, ip)) + em * lds<T>(d, L, im));
        const T t2 = lds<T>(d, M2[b], c) * (-(fp * lds<T>(d, L, jp)) + fm * lds<T>(d, L, jm));
        const T t3 = lds<T>(d, M3[b], c) * (-(gp * lds<T>(d, L, kp)) + gm * lds<T>(d, L, km));
        s = b == 0 ? t1 : s + t1;
        s = s + t2;
        s = s + t3;
    }
    return scale2(s, 0.5f);
}

// SGS divergence added to the advection terms (main.f90:59-69)
template <class T>
__global__ void k3_sgs(D3 d)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    const double *r0[3] = {d.L[0], d.L[1], d.L[2]}, *r1[3] = {d.L[3], d.L[4], d.L[5]}, *r2[3] = {d.L[6], d.L[7], d.L[8]};
    const T J = lds<T>(d, d.DJAC, c);
    d.NLX[c] = to_d(ld<T>(d.NLX[c]) + sgs_div<T>(d, d.EV, r0, i, j, k) * J);
    d.NLY[c] = to_d(ld<T>(d.NLY[c]) + sgs_div<T>(d, d.EV, r1, i, j, k) * J);
    d.NLZ[c] = to_d(ld<T>(d.NLZ[c]) + sgs_div<T>(d, d.EV, r2, i, j, k) * J);
}

template <class T>
__global__ void k3_sgst(D3 d)
{
    CELL3(1, d.NI - 1, 1, d.NJ - 1, 1, d.NK - 1)
    const int c = ID3(i, j, k);
    const double *g[3] = {d.DTD[0], d.DTD[1], d.DTD[2]};
    d.ADV[c] = to_d(ld<T>(d.ADV[c]) + sgs_div<T>(d, d.EC, g, i, j, k) * lds<T>(d, d.DJAC, c));
}

// ---------------------------------------------------------------------------------
// CALCCOEF (calccoef.f90:9-160)
// ---------------------------------------------------------------------------------
// CFL maximum: the maximum of the block (exact, order-free) goes to one atomic.
__global__ void __launch_bounds__(128) k3_cfl(D3 d)
{
    __shared__ double sh[4];
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
    double l = 0.0;
    if (i <= d.NI - 1) {
        const int c = ID3(i, j, k);
        const double u = d.U[c], v = d.V[c], w = d.W[c];
        l = d.dt * ((fabs((d.XIX[c] * u + d.XIY[c] * v) + d.XIZ[c] * w) +
                     fabs((d.ETX[c] * u + d.ETY[c] * v) + d.ETZ[c] * w)) +
                    fabs((d.ZTX[c] * u + d.ZTY[c] * v) + d.ZTZ[c] * w));
    }
    for (int o = 16; o > 0; o >>= 1) l = fmax(l, __shfl_xor_sync(0xffffffffu, l, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        const double m = fmax(fmax(sh[0], sh[1]), fmax(sh[2], sh[3]));
        atomicMax(d.cflbits, (unsigned long long)__double_as_longlong(m));
    }
}

// Wall force and heat-flux contributions of the two triangles of each wall face.
__global__ void k3_wall(D3 d)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1, tri = blockIdx.z;
    if (j > d.NJ - 1 || k > d.NK - 1) return;
    const int i = 1, c = ID3(i, j, k);
    int p, q, r;
    if (tri == 0) { p = ID3(i, j, k); q = ID3(i, j + 1, k); r = ID3(i, j, k + 1); }
    else { p = ID3(i, j + 1, k + 1); q = ID3(i, j, k + 1); r = ID3(i, j, k); }
    const double *XG = d.XG, *YG = d.YG, *ZG = d.ZG;
    const double A = (YG[p] * (ZG[q] - ZG[r]) + YG[q] * (ZG[r] - ZG[p])) + YG[r] * (ZG[p] - ZG[q]);
    const double B = (ZG[p] * (XG[q] - XG[r]) + ZG[q] * (XG[r] - XG[p])) + ZG[r] * (XG[p] - XG[q]);
    const double C = (XG[p] * (YG[q] - YG[r]) + XG[q] * (YG[r] - YG[p])) + XG[r] * (YG[p] - YG[q]);
    double D = (XG[p] * (YG[q] * ZG[r] - YG[r] * ZG[q]) + XG[q] * (YG[r] * ZG[p] - YG[p] * ZG[r])) +
               XG[r] * (YG[p] * ZG[q] - YG[q] * ZG[p]);
    D = -1.0 * D;
    const double dum = sqrt((A * A + B * B) + C * C);
    const double dn = fabs(((A * d.X[c] + B * d.Y[c]) + C * d.Z[c]) + D) / dum;
    const double u = d.U[c], v = d.V[c], w = d.W[c];
    const double e1 = (v * C) / dum - (w * B) / dum, e2 = (u * C) / dum - (w * A) / dum, e3 = (u * B) / dum - (v * A) / dum;
    double dudn = sqrt((e1 * e1 + e2 * e2) + e3 * e3);
    dudn = dudn / dn;
    const double area = tri == 0 ? d.AREA1[c] : d.AREA2[c];
    const double vm = sqrt((u * u + v * v) + w * w);
    double *o = d.wall + 8 * (size_t(tri) * d.NJ1 * (d.NK + 1) + JK(j, k));
    o[0] = (((2.0 * d.P[c]) * area) * A) / dum;
    o[1] = (((2.0 * d.P[c]) * area) * B) / dum;
    o[2] = ((((2.0 / d.re) * dudn) * area) * u) / vm;
    o[3] = ((((2.0 / d.re) * dudn) * area) * v) / vm;
    o[4] = ((d.T[c] - d.t_wall) / dn) * area;
}

// Sums of the wall contributions in a fixed tree (one block: a strided partial sum
// per thread, then the warps' shuffle trees, then the warps in order), the
// coefficients into scal[3..16].
__global__ void __launch_bounds__(1024) k3_calc_final(D3 d, double rtime, double sum_area)
{
    __shared__ double sh[5][32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int nj1 = d.NJ - 1, nk1 = d.NK - 1, plane = nj1 * nk1, total = 2 * plane;
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int e = t; e < total; e += blockDim.x) {
        const int tri = e / plane, r = e - tri * plane, k = r / nj1 + 1, j = r - (k - 1) * nj1 + 1;
        const double *o = d.wall + 8 * (size_t(tri) * d.NJ1 * (d.NK + 1) + JK(j, k));
        acc[0] = acc[0] - o[0];
        acc[1] = acc[1] - o[1];
        acc[2] = acc[2] + o[2];
        acc[3] = acc[3] + o[3];
        acc[4] = acc[4] + o[4];
    }
#pragma unroll
    for (int q = 0; q < 5; q++) {
        for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
        if (lane == 0) sh[q][warp] = acc[q];
    }
    __syncthreads();
    if (t != 0) return;
    double pd = 0.0, pl = 0.0, td = 0.0, tl = 0.0, snu = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        pd += sh[0][w];
        pl += sh[1][w];
        td += sh[2][w];
        tl += sh[3][w];
        snu += sh[4][w];
    }
    const double *P = d.P;
    double dumb = 0.0;
    for (int k = 1; k <= d.NK - 1; k++) {
        const int i = 1, j = 1;
        const double pg = 0.125 * (((((((P[ID3(i, j, k)] + P[ID3(i, j - 1, k)]) + P[ID3(i - 1, j, k)]) +
                                       P[ID3(i - 1, j - 1, k)]) + P[ID3(i, j, k + 1)]) + P[ID3(i, j - 1, k + 1)]) +
                                     P[ID3(i - 1, j, k + 1)]) + P[ID3(i - 1, j - 1, k + 1)]);
        dumb = dumb + pg;
    }
    dumb = dumb / (double)(d.NK - 1);
    double *s = d.scal + 3;
    s[0] = rtime;
    s[1] = __longlong_as_double((long long)*d.cflbits);
    s[2] = 0.0 + 2.0 * (0.0 - dumb);
    s[5] = pd / d.ref_a;
    s[7] = pl / d.ref_a;
    s[6] = td / d.ref_a;
    s[8] = tl / d.ref_a;
    s[3] = s[5] + s[6];
    s[4] = s[7] + s[8];
    s[9] = -snu / sum_area;
    s[10] = d.scal[0];
    s[11] = d.scal[1];
    s[12] = (double)d.pctl->niter;
    s[13] = d.pctl->resip;
    *d.cflbits = 0ull;
}

}  // namespace f3

namespace f3 {
// The post-processing block of CALCCOEF (calccoef.f90:286-307): the step added to
// the sums of U, V, W, P, T (ps 0..4), of the six velocity products (5..10) and of
// the SGS stresses -2 nu_t S_ij of the step's model (11..16), over the whole array.
__global__ void k3_post_acc(D3 d, double *ps)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const size_t n = d.n;
    const double u = d.U[c], v = d.V[c], w = d.W[c], f[3] = {u, v, w};
    ps[c] += u;
    ps[n + c] += v;
    ps[2 * n + c] += w;
    ps[3 * n + c] += d.P[c];
    ps[4 * n + c] += d.T[c];
    const int ra[6] = {0, 0, 0, 1, 1, 2}, rb[6] = {0, 1, 2, 1, 2, 2}, ls[6] = {0, 1, 2, 4, 5, 8};
#pragma unroll
    for (int q = 0; q < 6; q++) ps[(5 + q) * n + c] += f[ra[q]] * f[rb[q]];
    const double ev2 = 2.0 * d.EV[c];
#pragma unroll
    for (int q = 0; q < 6; q++) ps[(11 + q) * n + c] -= ev2 * d.L[ls[q]][c];
}
}  // namespace f3

// ---------------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------------
struct fvm3_ctx {
    fvm3_params p{};
    int NI = 0, NJ = 0, NK = 0, n = 0;
    cudaStream_t stream = nullptr;
    f3::D3 d{};
    char *slab = nullptr;
    std::string err;
    bool grid_set = false, init_done = false;
    double rtime = 0.0, sum_area = 0.0;
    int niter_time = 0;
    fvm::PCtl *h_pctl = nullptr;
    cudaGraphExec_t pgraph = nullptr;
    int pgraph_iters = 0;
    fvm3_coeffs last{};
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    // post-processing: 17 sum arrays on the device, allocated on first use
    double *post = nullptr;
    int ipost = 0, niter_pos = 0;
    // the shadowed group's address range (arrays with (hi, lo) shadows in the mixed path)
    double *shadow_lo = nullptr, *shadow_hi = nullptr;
};

namespace f3 {
namespace {

#define F3CUDA(c, call)                                                            \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            (c)->err = std::string(#call) + ": " + cudaGetErrorString(e_);         \
            return FVM_ERR_CUDA;                                                   \
        }                                                                          \
    } while (0)
#define F3CHECK(c)                                                                 \
    do {                                                                           \
        cudaError_t e_ = cudaGetLastError();                                       \
        if (e_ != cudaSuccess) {                                                   \
            (c)->err = std::string("kernel launch: ") + cudaGetErrorString(e_);    \
            return FVM_ERR_CUDA;                                                   \
        }                                                                          \
    } while (0)
#define F3RC(x)               \
    do {                      \
        int rc_ = (x);        \
        if (rc_) return rc_;  \
    } while (0)

struct Bump {
    char *base;
    size_t off = 0;
    double *take(size_t count)
    {
        off = (off + 255) & ~size_t(255);
        double *p = base ? reinterpret_cast<double *>(base + off) : nullptr;
        off += count * sizeof(double);
        return p;
    }
};

void carve(Bump &b, fvm3_ctx *c)
{
    D3 &d = c->d;
    const size_t n = c->n, jk = size_t(c->NJ + 1) * (c->NK + 1);
    // The shadowed group: the arrays the double-float kernels of the mixed path read
    // through (hi, lo) shadows.  Taken consecutively with equal sizes, so that in the
    // mixed path a second block taken in the same order puts every shadow at the
    // same element offset sh from its array.
    std::vector<double **> grp = {&d.XIX, &d.XIY, &d.XIZ, &d.ETX, &d.ETY, &d.ETZ, &d.ZTX, &d.ZTY, &d.ZTZ, &d.DJAC,
                                  &d.FW, &d.DE, &d.DW, &d.DN, &d.DS, &d.DT, &d.DB, &d.U, &d.V, &d.W, &d.T,
                                  &d.U_N, &d.V_N, &d.W_N, &d.T_N, &d.MAG, &d.UH, &d.VH, &d.WH, &d.TH, &d.EV, &d.EC};
    for (int q = 0; q < 9; q++) grp.push_back(&d.L[q]);
    for (int q = 0; q < 3; q++) grp.push_back(&d.DTD[q]);
    for (int e = 0; e < 12; e++) grp.push_back(&d.CW[e]);
    for (int sp = 0; sp < 3; sp++)
        for (int e = 0; e < 12; e++) grp.push_back(&d.CWA[sp][e]);
    for (int st = 0; st < 6; st++) {   // the couplings of the predictor sets
        Coef3 &cf = d.cf[st];
        for (double **p : {&cf.AE, &cf.AW, &cf.AN, &cf.AS, &cf.AT, &cf.AB}) grp.push_back(p);
    }
    for (auto p : grp) *p = b.take(n);
    d.dfl = c->p.precision == FVM_MIXED ? 1 : 0;
    d.sh = 0;
    if (d.dfl) {
        double *first = nullptr;
        for (size_t q = 0; q < grp.size(); q++) {
            double *t = b.take(n);
            if (q == 0) first = t;
        }
        d.sh = b.base ? (long long)(first - d.XIX) : 0;
    }
    if (b.base) {
        c->shadow_lo = d.XIX;
        c->shadow_hi = *grp.back() + n;
    }
    double **full[] = {&d.XG, &d.YG, &d.ZG, &d.X, &d.Y, &d.Z, &d.Q11, &d.Q12, &d.Q13, &d.Q22, &d.Q23, &d.Q33,
                       &d.JQ12, &d.JQ13, &d.JQ23, &d.THETA, &d.AREA1, &d.AREA2, &d.P, &d.NLX, &d.NLY, &d.NLZ,
                       &d.ADV, &d.NLX_NM1, &d.NLY_NM1, &d.NLZ_NM1, &d.ADV_NM1, &d.DIFX, &d.DIFY, &d.DIFZ, &d.DIFT,
                       &d.S_U, &d.S_V, &d.S_W, &d.U1, &d.U2, &d.U3, &d.UE, &d.UW, &d.VN, &d.VS, &d.WT, &d.WB,
                       &d.DIVDT, &d.SU, &d.MAGH, &d.LM, &d.MM};
    for (auto p : full) *p = b.take(n);
    for (int q = 0; q < 9; q++) d.MD[q] = d.L[q];   // metric derivatives live in the strain arrays at setup
    double **perjk[] = {&d.FFU, &d.FFV, &d.FFW, &d.FFT};
    for (auto p : perjk) *p = b.take(jk);
    d.CZ = b.take(size_t(c->NI + 1) * (c->NJ + 1));
    for (int s = 0; s < 7; s++) {
        Coef3 &cf = d.cf[s];
        cf.AP = b.take(n);
        if (s == 6)
            for (double **p : {&cf.AE, &cf.AW, &cf.AN, &cf.AS, &cf.AT, &cf.AB}) *p = b.take(n);
        cf.awall = b.take(jk);
        cf.afar = b.take(jk);
    }
    // line families of the sets: 0,3,6 I lines; 1,4 J lines (cyclic); 2,5 K lines (cyclic)
    for (int s = 0; s < 7; s++) {
        const int fam = s == 6 ? 0 : s % 3;
        Fam F = family(fam, c->NI, c->NJ, c->NK);
        LineSys &ls = d.sys[s];
        ls.lines = F.lines;
        ls.n = F.n;
        ls.NW = fvm::group_warps(F.n);
        ls.M = (F.n + WARP * ls.NW - 1) / (WARP * ls.NW);
        if (fam == 0 && F.n > 128 && F.n <= 192) {   // one warp of 6 per thread: measured faster on the I lines
            ls.NW = 1;
            ls.M = 6;
        }
        if (fam == 0 && c->p.tile_i_warps > 0) {   // validated in fvm3_create
            ls.NW = c->p.tile_i_warps;
            ls.M = c->p.tile_i_m;
        }
        ls.cyclic = fam != 0;
        const size_t cnt = size_t(F.lines) * WARP * ls.NW * ls.M;
        ls.invD = b.take(cnt);
        ls.fa = b.take(cnt);
        ls.fb = b.take(cnt);
        ls.invDf = reinterpret_cast<float *>(b.take((cnt + 1) / 2));
        ls.faf = reinterpret_cast<float *>(b.take((cnt + 1) / 2));
        ls.fbf = reinterpret_cast<float *>(b.take((cnt + 1) / 2));
        if (ls.cyclic) {
            ls.z = b.take(cnt);
            ls.zf = reinterpret_cast<float *>(b.take((cnt + 1) / 2));
            ls.cv = b.take(F.lines);
            ls.sinv = b.take(F.lines);
            ls.cvf = reinterpret_cast<float *>(b.take(F.lines));
            ls.sinvf = reinterpret_cast<float *>(b.take(F.lines));
        }
        if (s < 6 && d.dfl) {
            LineDD &sd = d.sysd[s];
            sd.invD = reinterpret_cast<dd *>(b.take(cnt));
            sd.fa = reinterpret_cast<dd *>(b.take(cnt));
            sd.fb = reinterpret_cast<dd *>(b.take(cnt));
            sd.z = ls.cyclic ? reinterpret_cast<dd *>(b.take(cnt)) : nullptr;
            sd.cv = ls.cyclic ? reinterpret_cast<dd *>(b.take(F.lines)) : nullptr;
            sd.sinv = ls.cyclic ? reinterpret_cast<dd *>(b.take(F.lines)) : nullptr;
        }
    }
    float **f32[] = {&d.RF, &d.DF, &d.ANf, &d.ATf};
    for (auto p : f32) *p = reinterpret_cast<float *>(b.take((n + 1) / 2));
    d.FB = b.take(24 * n);
    d.nblk = 8 * 152;   // residual and reduction kernels: 8 blocks of 256 threads per SM
    d.partial = b.take(4 * size_t(d.nblk));
    d.pctl = reinterpret_cast<PCtl *>(b.take(8));
    d.scal = b.take(32);
    d.cflbits = reinterpret_cast<unsigned long long *>(b.take(1));
    d.wall = b.take(16 * jk);
}

// Interior launches: 32 x 4 blocks in (I, J), one K plane per grid z.
inline dim3 g_int(const fvm3_ctx *c) { return dim3((c->NI - 1 + 31) / 32, (c->NJ - 1 + 3) / 4, c->NK - 1); }
const dim3 B_INT(32, 4, 1);
inline dim3 g_full3(const fvm3_ctx *c) { return dim3((c->NI + 1 + 127) / 128, c->NJ + 1, c->NK + 1); }
inline int g_lin(const fvm3_ctx *c) { return (c->n + 255) / 256; }

int halo(fvm3_ctx *c, std::initializer_list<double *> arrs)
{
    Arrs A{};
    A.n = 0;
    for (double *a : arrs) A.a[A.n++] = a;
    k3_halo<<<dim3((c->NI + 1 + 127) / 128, c->NK + 1 + c->NJ + 1), 128, 0, c->stream>>>(c->d, A);
    F3CHECK(c);
    return FVM_OK;
}

// Periodic copy of the shadows of shadowed arrays (mixed path).
int halo_shadows(fvm3_ctx *c, const std::vector<double *> &arrs)
{
    if (!c->d.dfl) return FVM_OK;
    Arrs A{};
    A.n = 0;
    for (double *a : arrs) A.a[A.n++] = a + c->d.sh;
    k3_halo<<<dim3((c->NI + 1 + 127) / 128, c->NK + 1 + c->NJ + 1), 128, 0, c->stream>>>(c->d, A);
    F3CHECK(c);
    return FVM_OK;
}

// Refresh the shadows of shadowed arrays from their doubles (mixed path; a no-op
// in the FP64 path).
int refresh(fvm3_ctx *c, const std::vector<double *> &arrs)
{
    if (!c->d.dfl) return FVM_OK;
    Arrs A{};
    A.n = 0;
    for (size_t q = 0; q < arrs.size(); q++) {
        A.a[A.n++] = arrs[q];
        if (A.n == 16 || q + 1 == arrs.size()) {
            k3_shadow<<<(c->n + 255) / 256, 256, 0, c->stream>>>(c->d, A);
            A.n = 0;
        }
    }
    F3CHECK(c);
    return FVM_OK;
}

// The geometry-only arrays of the shadowed group, after the setup.
int refresh_constants(fvm3_ctx *c)
{
    D3 &d = c->d;
    std::vector<double *> a = {d.XIX, d.XIY, d.XIZ, d.ETX, d.ETY, d.ETZ, d.ZTX, d.ZTY, d.ZTZ, d.DJAC, d.FW,
                               d.DE, d.DW, d.DN, d.DS, d.DT, d.DB};
    for (int e = 0; e < 12; e++) a.push_back(d.CW[e]);
    for (int sp = 0; sp < 3; sp++)
        for (int e = 0; e < 12; e++) a.push_back(d.CWA[sp][e]);
    for (int st = 0; st < 6; st++)
        for (double *p : {d.cf[st].AE, d.cf[st].AW, d.cf[st].AN, d.cf[st].AS, d.cf[st].AT, d.cf[st].AB}) a.push_back(p);
    return refresh(c, a);
}

int line(fvm3_ctx *c, int set, const double *SU, double *phi, int colour, const PCtl *stop = nullptr)
{
    const D3 &d = c->d;
    const LineSys &s = d.sys[set];
    const int fam = set == 6 ? 0 : set % 3;
    int per;
    if (fam == 0) per = (c->NJ - 1) / 2 * (c->NK - 1);
    else if (fam == 1) per = (c->NI - 1) * ((c->NK - 1) / 2);
    else per = (c->NI - 1) * ((c->NJ - 1) / 2);
    const int blocks = fvm::line_blocks(per, s.NW);
    bool ok = fvm::dispatch_line(s, [&](auto m, auto nw) {
        constexpr int M = decltype(m)::value, NW = decltype(nw)::value;
        const LineDD none{};
        if (d.dfl && set < 6) {   // predictor sets of the mixed path: double-float
            const LineDD &sd = d.sysd[set];
            if (fam == 0) k3_line<M, NW, 0, dd><<<blocks, 128, 0, c->stream>>>(d, s, d.cf[set], SU, phi, colour, stop, sd);
            else if (fam == 1) k3_line<M, NW, 1, dd><<<blocks, 128, 0, c->stream>>>(d, s, d.cf[set], SU, phi, colour, stop, sd);
            else k3_line<M, NW, 2, dd><<<blocks, 128, 0, c->stream>>>(d, s, d.cf[set], SU, phi, colour, stop, sd);
        } else if (fam == 0) {
            k3_line<M, NW, 0><<<blocks, 128, 0, c->stream>>>(d, s, d.cf[set], SU, phi, colour, stop, none);
        } else if (fam == 1) {
            k3_line<M, NW, 1><<<blocks, 128, 0, c->stream>>>(d, s, d.cf[set], SU, phi, colour, stop, none);
        } else {
            k3_line<M, NW, 2><<<blocks, 128, 0, c->stream>>>(d, s, d.cf[set], SU, phi, colour, stop, none);
        }
    });
    if (!ok) {
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    F3CHECK(c);
    return FVM_OK;
}

int line32(fvm3_ctx *c, int colour, int check_done, int apply)
{
    const D3 &d = c->d;
    const LineSys &s = d.sys[6];
    const int per = (c->NJ - 1) / 2 * (c->NK - 1);
    const int blocks = fvm::line_blocks(per, s.NW);
    bool ok = fvm::dispatch_line(s, [&](auto m, auto nw) {
        constexpr int M = decltype(m)::value, NW = decltype(nw)::value;
        k3_line32<M, NW><<<blocks, 128, 0, c->stream>>>(d, s, colour, check_done, apply);
    });
    if (!ok) {
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    F3CHECK(c);
    return FVM_OK;
}

int setup_grid(fvm3_ctx *c)
{
    D3 &d = c->d;
    cudaStream_t st = c->stream;
    k3_centres<<<g_full3(c), 128, 0, st>>>(d);
    k3_faces<<<g_full3(c), 128, 0, st>>>(d);
    F3RC(halo(c, {d.X, d.Y, d.Z}));
    k3_kplanes_xy_zin<<<dim3((c->NI + 1 + 127) / 128, c->NJ + 1, 2), 128, 0, st>>>(d);
    k3_kplanes_zedge<<<dim3((std::max(c->NI, c->NJ) + 127) / 128, 2), 128, 0, st>>>(d);
    k3_kplanes_zcorner<<<1, 32, 0, st>>>(d);
    k3_derivs<<<g_full3(c), 128, 0, st>>>(d);
    F3RC(halo(c, {d.MD[0], d.MD[1], d.MD[2], d.MD[3], d.MD[4], d.MD[5], d.MD[6], d.MD[7], d.MD[8]}));
    k3_jacobian<<<g_lin(c), 256, 0, st>>>(d);
    k3_q<<<g_lin(c), 256, 0, st>>>(d);
    k3_dcoef<<<g_int(c), B_INT, 0, st>>>(d);
    k3_theta<<<g_lin(c), 256, 0, st>>>(d);
    k3_areas<<<dim3((c->NJ + 127) / 128, c->NK - 1), 128, 0, st>>>(d);
    for (int s = 0; s < 3; s++) {
        k3_coef_af<<<g_int(c), B_INT, 0, st>>>(d, d.cf[s], s, d.re);
        k3_coef_af<<<g_int(c), B_INT, 0, st>>>(d, d.cf[3 + s], s, d.pe);
    }
    k3_coef_p<<<g_int(c), B_INT, 0, st>>>(d, d.cf[6]);
    for (int set = -1; set < 3; set++) k3_cw<<<g_int(c), B_INT, 0, st>>>(d, set);
    k3_coef_f32<<<g_lin(c), 256, 0, st>>>(d);
    F3CHECK(c);
    for (int s = 0; s < 7; s++) {
        const int fam = s == 6 ? 0 : s % 3;
        k3_factor<<<(d.sys[s].lines + 63) / 64, 64, 0, st>>>(d, d.cf[s], d.sys[s], fam, fam != 0);
    }
    if (d.dfl)
        for (int s = 0; s < 6; s++) {
            const LineSys &ls = d.sys[s];
            const size_t cnt = size_t(ls.lines) * WARP * ls.NW * ls.M;
            k3_factor_dd<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(ls, d.sysd[s], cnt);
        }
    F3CHECK(c);
    F3RC(refresh_constants(c));
    // sum of the wall areas in the reference's loop order (init.f90:186-190)
    std::vector<double> a1(c->n), a2(c->n), dj(c->n);
    F3CUDA(c, cudaMemcpyAsync(a1.data(), d.AREA1, sizeof(double) * c->n, cudaMemcpyDeviceToHost, st));
    F3CUDA(c, cudaMemcpyAsync(a2.data(), d.AREA2, sizeof(double) * c->n, cudaMemcpyDeviceToHost, st));
    F3CUDA(c, cudaMemcpyAsync(dj.data(), d.DJAC, sizeof(double) * c->n, cudaMemcpyDeviceToHost, st));
    F3CUDA(c, cudaStreamSynchronize(st));
    double dum = 0.0;
    const int NI1 = c->NI + 1, NJ1 = c->NJ + 1;
    for (int k = 1; k <= c->NK - 1; k++)
        for (int j = 1; j <= c->NJ - 1; j++) {
            const int q = 1 + NI1 * (j + NJ1 * k);
            dum = (dum + a1[q]) + a2[q];
        }
    c->sum_area = dum;
    for (int q = 0; q < c->n; q++)
        if (!(std::fabs(dj[q]) >= 1e-15)) {
            c->err = "grid has a cell with |Jacobian| < 1e-15";
            return FVM_ERR_ARG;
        }
    return FVM_OK;
}

// The stencils of the SGS model, DIF, NL, P_SOURCE and the AF right-hand sides run
// in double-float in the mixed path (FP64 in memory) and in FP64 otherwise.
static inline bool dfloat(const fvm3_ctx *c) { return c->p.precision == FVM_MIXED; }
#define F3_LAUNCH(c, K, grid, block, ...)                                         \
    do {                                                                          \
        if (dfloat(c)) K<dd><<<(grid), (block), 0, (c)->stream>>>(__VA_ARGS__);   \
        else K<double><<<(grid), (block), 0, (c)->stream>>>(__VA_ARGS__);         \
    } while (0)

int bcu(fvm3_ctx *c, double *phi, const double *ff, int kind);

// One predictor sweep set (three AF sweeps) of a field: kind 0 U, 1 V or W, 2 T.
int predictor(fvm3_ctx *c, int kind, double *phi, const double *phin, const double *ina, const double *inb,
              const double *inc, const double *ind, const double *ff)
{
    D3 &d = c->d;
    const int base = kind == 2 ? 3 : 0;
    // the field's shadow: refreshed once; later the line solves write the interior
    // shadows and k3_bcu the ghosts'
    F3RC(refresh(c, {phi}));
    for (int split = 0; split < 3; split++) {
        F3_LAUNCH(c, k3_af_rhs, g_int(c), B_INT, d, d.cf[base + split], split, kind, phi, phin, ina, inb, inc, ind,
                  ff);
        F3RC(bcu(c, phi, ff, kind));
        F3RC(line(c, base + split, d.SU, phi, 0));
        F3RC(line(c, base + split, d.SU, phi, 1));
    }
    return FVM_OK;
}

int bcu(fvm3_ctx *c, double *phi, const double *ff, int kind)
{
    const long long nt = (long long)(c->NJ - 1) * (c->NK - 1) +
                         (2LL * (c->NJ + 1) + 2LL * (c->NK - 1)) * (c->NI + 1);
    k3_bcu<<<(unsigned)((nt + 255) / 256), 256, 0, c->stream>>>(c->d, phi, ff, kind);
    F3CHECK(c);
    return FVM_OK;
}

// The Poisson loop body: `groups` x (res_every x [source, BCP, sweep], residual).
int poisson_graph(fvm3_ctx *c)
{
    if (c->pgraph) return FVM_OK;
    D3 &d = c->d;
    const bool mixed = c->p.precision == FVM_MIXED;
    const int per = mixed ? d.refine_sweeps : d.res_every, groups = std::max(1, 32 / per);
    // host loop: the graph is one body, replayed until the control block reports
    // completion; device loop: a while node whose condition the residual kernel
    // clears when the iteration has converged or reached the cap
    const int dev_loop = c->p.poisson_host_loop ? 0 : 1;
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle h = 0;
    cudaGraphNodeParams cp = {};
    cudaError_t e = cudaSuccess;
    if (dev_loop) {
        F3CUDA(c, cudaGraphCreate(&g, 0));
        e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(c->stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
    } else {
        e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    }
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        c->err = std::string("Poisson loop node: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    int rc = FVM_OK;
    for (int q = 0; q < groups && rc == FVM_OK && mixed; q++) {
        // residual (ends the loop), FP32 correction sweeps, P += dP, ghosts
        if (dev_loop) k3_mres<1><<<d.nblk, 256, 0, c->stream>>>(d, h);
        else k3_mres<0><<<d.nblk, 256, 0, c->stream>>>(d, h);
        for (int it = 0; it < per && rc == FVM_OK; it++) {
            rc = line32(c, 0, 1, 0);
            if (rc == FVM_OK) rc = line32(c, 1, 1, it == per - 1);   // the last one adds dP and the BCP ghosts
        }
        if (rc == FVM_OK) rc = halo(c, {d.P});
    }
    for (int q = 0; q < groups && rc == FVM_OK && !mixed; q++) {
        for (int it = 0; it < per && rc == FVM_OK; it++) {
            k3_psu<<<g_int(c), B_INT, 0, c->stream>>>(d);
            k3_bcp<<<dim3((c->NJ + 127) / 128, c->NK + 1), 128, 0, c->stream>>>(d, 1);
            rc = halo(c, {d.P});
            if (rc == FVM_OK) rc = line(c, 6, d.SU, d.P, 0, d.pctl);
            if (rc == FVM_OK) rc = line(c, 6, d.SU, d.P, 1, d.pctl);
        }
        if (dev_loop) k3_pres<1><<<d.nblk, 256, 0, c->stream>>>(d, d.cf[6], per, h);
        else k3_pres<0><<<d.nblk, 256, 0, c->stream>>>(d, d.cf[6], per, h);
    }
    cudaGraph_t body = dev_loop ? cp.conditional.phGraph_out[0] : nullptr;
    e = cudaStreamEndCapture(c->stream, &body);
    if (!dev_loop) g = body;
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (!rc) c->err = std::string("Poisson capture: ") + cudaGetErrorString(e);
        return rc ? rc : FVM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&c->pgraph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->err = std::string("Poisson instantiate: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    c->pgraph_iters = per * groups;
    return FVM_OK;
}

int poisson(fvm3_ctx *c)
{
    D3 &d = c->d;
    F3RC(poisson_graph(c));
    k3_pctl_reset<<<1, 1, 0, c->stream>>>(d);
    if (!c->p.poisson_host_loop) {
        // one launch: the loop runs on the device until the residual kernel ends it
        // (the sweep cap bounds it); the statistics stay on the device for CALCCOEF
        F3CUDA(c, cudaGraphLaunch(c->pgraph, c->stream));
        return FVM_OK;
    }
    const long max_launches = (long)d.nswpp / c->pgraph_iters + 2;
    for (long l = 0;; l++) {
        if (l >= max_launches) {
            c->err = "Poisson iteration did not report completion within the sweep cap";
            return FVM_ERR_TIMEOUT;
        }
        F3CUDA(c, cudaGraphLaunch(c->pgraph, c->stream));
        F3CUDA(c, cudaMemcpyAsync(c->h_pctl, d.pctl, sizeof(PCtl), cudaMemcpyDeviceToHost, c->stream));
        F3CUDA(c, cudaStreamSynchronize(c->stream));
        if (c->h_pctl->done) break;
    }
    return FVM_OK;
}

// The separable test filter of the inputs of `mode` (SEP_HATS: into UH, VH, WH,
// TH; otherwise into bank 1).
int sep_filter(fvm3_ctx *c, int mode)
{
    D3 &d = c->d;
    const int nq = mode == SEP_HATS ? 4 : (mode == SEP_VEL ? 12 : 6);
    Out4 none{}, hats{};
    if (mode == SEP_HATS) hats = Out4{{d.UH, d.VH, d.WH, d.TH}};
    F3_LAUNCH(c, k3_prod, g_lin(c), 256, d, mode);
    const dim3 gi((c->NI - 1 + 31) / 32, (c->NJ + 1 + 3) / 4, c->NK + 1), gj((c->NI - 1 + 31) / 32, (c->NJ - 1 + 3) / 4, c->NK + 1);
    F3_LAUNCH(c, k3_sep, gi, B_INT, d, 0, 1, nq, 0, none);
    F3_LAUNCH(c, k3_sep, gj, B_INT, d, 1, 0, nq, 1, none);
    F3_LAUNCH(c, k3_sep, g_int(c), B_INT, d, 0, 1, nq, 2, mode == SEP_HATS ? hats : none);
    F3CHECK(c);
    return FVM_OK;
}

int sgs(fvm3_ctx *c)
{
    D3 &d = c->d;
    cudaStream_t st = c->stream;
    const dim3 gs((c->NI + 1 + 31) / 32, (c->NJ - 1 + 3) / 4, c->NK - 1);
    F3RC(refresh(c, {d.U, d.V, d.W, d.T}));
    F3_LAUNCH(c, k3_strain, gs, B_INT, d);   // L and DTD with their shadows
    F3RC(halo(c, {d.L[0], d.L[1], d.L[2], d.L[3], d.L[4], d.L[5], d.L[6], d.L[7], d.L[8], d.DTD[0], d.DTD[1],
                  d.DTD[2]}));
    F3RC(halo_shadows(c, {d.L[0], d.L[1], d.L[2], d.L[3], d.L[4], d.L[5], d.L[6], d.L[7], d.L[8], d.DTD[0],
                          d.DTD[1], d.DTD[2]}));
    F3_LAUNCH(c, k3_mag, g_lin(c), 256, d);
    F3RC(sep_filter(c, SEP_HATS));
    F3RC(bcu(c, d.UH, d.FFU, 0));
    F3RC(bcu(c, d.VH, d.FFV, 1));
    F3RC(bcu(c, d.WH, d.FFW, 1));
    F3RC(bcu(c, d.TH, d.FFT, 2));
    F3RC(refresh(c, {d.UH, d.VH, d.WH, d.TH}));
    F3RC(sep_filter(c, SEP_VEL));
    F3_LAUNCH(c, k3_germano, g_int(c), B_INT, d, 1);
    if (d.les_zavg) k3_czavg<<<dim3((c->NI - 1 + 127) / 128, c->NJ - 1), 128, 0, st>>>(d);
    else k3_cvol<<<d.nblk, 256, 0, st>>>(d, 0);
    k3_eddy<<<g_lin(c), 256, 0, st>>>(d, 0, d.EV);
    F3_LAUNCH(c, k3_sgs, g_int(c), B_INT, d);
    if (d.thermal) {
        F3RC(sep_filter(c, SEP_HEAT));
        F3_LAUNCH(c, k3_germano_t, g_int(c), B_INT, d, 1);
        if (d.les_zavg) k3_czavg<<<dim3((c->NI - 1 + 127) / 128, c->NJ - 1), 128, 0, st>>>(d);
        else k3_cvol<<<d.nblk, 256, 0, st>>>(d, 1);
        k3_eddy<<<g_lin(c), 256, 0, st>>>(d, 1, d.EC);
        F3_LAUNCH(c, k3_sgst, g_int(c), B_INT, d);
    }
    F3CHECK(c);
    return FVM_OK;
}

int read_coeffs(fvm3_ctx *c, fvm3_coeffs *out)
{
    double s[14];
    F3CUDA(c, cudaMemcpyAsync(s, c->d.scal + 3, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    fvm3_coeffs co;
    co.time = s[0]; co.cfl = s[1]; co.cpb = s[2]; co.cd = s[3]; co.cl = s[4]; co.cd_p = s[5]; co.cd_v = s[6];
    co.cl_p = s[7]; co.cl_v = s[8]; co.nu = s[9]; co.cs2 = s[10]; co.ct2 = s[11]; co.sweeps = (int)s[12];
    co.resid = s[13];
    c->last = co;
    if (out) *out = co;
    if (!std::isfinite(co.cd) || !std::isfinite(co.resid)) {
        c->err = "non-finite drag or Poisson residual";
        return FVM_ERR_NAN;
    }
    return FVM_OK;
}

// The routines of the time loop (main.f90:33-147), one host function per call point.
int begin_step(fvm3_ctx *c)   // main.f90:37-44, the far-field values of BCU/BCT from the step-n fields
{
    D3 &d = c->d;
    c->niter_time += 1;
    c->rtime = c->rtime + d.dt;
    k3_begin<<<g_lin(c), 256, 0, c->stream>>>(d);
    k3_farfield<<<dim3((c->NJ + 127) / 128, c->NK - 1), 128, 0, c->stream>>>(d);
    F3CHECK(c);
    return refresh(c, {d.U_N, d.V_N, d.W_N, d.T_N});
}

int contra_vel(fvm3_ctx *c, int with_div)   // CONTRA_VEL; with_div: the Poisson source too
{
    D3 &d = c->d;
    k3_contra<<<g_lin(c), 256, 0, c->stream>>>(d);
    F3RC(halo(c, {d.U1, d.U2, d.U3}));
    k3_fluxes<<<g_int(c), B_INT, 0, c->stream>>>(d, with_div);
    F3CHECK(c);
    return FVM_OK;
}

int nl_all(fvm3_ctx *c)   // main.f90:50-57
{
    F3_LAUNCH(c, k3_explicit, g_int(c), B_INT, c->d, c->d.thermal);
    F3CHECK(c);
    return FVM_OK;
}

int dif_all(fvm3_ctx *c)   // main.f90:72-75
{
    F3_LAUNCH(c, k3_dif, g_int(c), B_INT, c->d, c->d.thermal);
    F3CHECK(c);
    return FVM_OK;
}

int p_source(fvm3_ctx *c)   // P_SOURCE(P)
{
    F3_LAUNCH(c, k3_psource, g_int(c), B_INT, c->d);
    F3CHECK(c);
    return FVM_OK;
}

int iter_u(fvm3_ctx *c, int comp)   // ITER_U of U (0), V (1) or W (2), main.f90:81-88
{
    D3 &d = c->d;
    if (comp == 0) return predictor(c, 0, d.U, d.U_N, d.NLX, d.NLX_NM1, d.DIFX, d.S_U, d.FFU);
    if (comp == 1) return predictor(c, 1, d.V, d.V_N, d.NLY, d.NLY_NM1, d.DIFY, d.S_V, d.FFV);
    return predictor(c, 1, d.W, d.W_N, d.NLZ, d.NLZ_NM1, d.DIFZ, d.S_W, d.FFW);
}

int bcu_all(fvm3_ctx *c)   // BCU of U, V, W
{
    D3 &d = c->d;
    F3RC(bcu(c, d.U, d.FFU, 0));
    F3RC(bcu(c, d.V, d.FFV, 1));
    F3RC(bcu(c, d.W, d.FFW, 1));
    return FVM_OK;
}

int remove_grad(fvm3_ctx *c)   // main.f90:90-97: u -= dt S/J, BCU
{
    F3_LAUNCH(c, k3_grad, g_int(c), B_INT, c->d, -1.0);
    F3CHECK(c);
    return bcu_all(c);
}

int iter_p(fvm3_ctx *c)   // main.f90:99-104: CONTRA_VEL, ITER_P, BCP
{
    D3 &d = c->d;
    F3RC(contra_vel(c, 1));
    F3RC(poisson(c));
    k3_bcp<<<dim3((c->NJ + 127) / 128, c->NK + 1), 128, 0, c->stream>>>(d, 0);
    F3RC(halo(c, {d.P}));
    return FVM_OK;
}

int correct(fvm3_ctx *c)   // main.f90:106-140: P_SOURCE, u += dt S/J, reference pressure, BCU
{
    D3 &d = c->d;
    F3_LAUNCH(c, k3_psource, g_int(c), B_INT, d);
    F3_LAUNCH(c, k3_grad, g_int(c), B_INT, d, +1.0);
    k3_pref<<<1, 32, 0, c->stream>>>(d);
    k3_pshift<<<g_lin(c), 256, 0, c->stream>>>(d);
    F3CHECK(c);
    return bcu_all(c);
}

int iter_t(fvm3_ctx *c)   // main.f90:143-145: ITER_T, BCT
{
    D3 &d = c->d;
    if (!d.thermal) return FVM_OK;
    F3RC(predictor(c, 2, d.T, d.T_N, d.ADV, d.ADV_NM1, d.DIFT, nullptr, d.FFT));
    return bcu(c, d.T, d.FFT, 2);
}

int calccoef(fvm3_ctx *c)   // CALCCOEF kernels; the record is read by read_coeffs
{
    D3 &d = c->d;
    k3_cfl<<<dim3((c->NI - 1 + 127) / 128, c->NJ - 1, c->NK - 1), 128, 0, c->stream>>>(d);
    k3_wall<<<dim3((c->NJ + 127) / 128, c->NK - 1, 2), 128, 0, c->stream>>>(d);
    k3_calc_final<<<1, 1024, 0, c->stream>>>(d, c->rtime, c->sum_area);
    if (c->ipost && c->post) {
        k3_post_acc<<<g_lin(c), 256, 0, c->stream>>>(d, c->post);
        c->niter_pos += 1;
    }
    F3CHECK(c);
    return FVM_OK;
}

int step(fvm3_ctx *c)
{
    F3RC(begin_step(c));
    F3RC(contra_vel(c, 0));
    F3RC(nl_all(c));
    if (c->p.use_les) F3RC(sgs(c));
    F3RC(dif_all(c));
    F3RC(p_source(c));
    for (int comp = 0; comp < 3; comp++) F3RC(iter_u(c, comp));
    F3RC(remove_grad(c));
    F3RC(iter_p(c));
    F3RC(correct(c));
    F3RC(iter_t(c));
    return calccoef(c);
}

double *array_by_name(fvm3_ctx *c, const char *name)
{
    D3 &d = c->d;
    struct { const char *n; double *a; } t[] = {
        {"U", d.U}, {"V", d.V}, {"W", d.W}, {"P", d.P}, {"T", d.T}, {"NLX", d.NLX}, {"NLY", d.NLY}, {"NLZ", d.NLZ},
        {"ADV", d.ADV}, {"X", d.X}, {"Y", d.Y}, {"Z", d.Z}, {"DJAC", d.DJAC}, {"XIX", d.XIX}, {"XIY", d.XIY},
        {"XIZ", d.XIZ}, {"ETX", d.ETX}, {"ETY", d.ETY}, {"ETZ", d.ETZ}, {"ZTX", d.ZTX}, {"ZTY", d.ZTY},
        {"ZTZ", d.ZTZ}, {"DE", d.DE}, {"DN", d.DN}, {"DT", d.DT}, {"THETA", d.THETA}, {"EDDY_VISCOS", d.EV},
        {"MAG", d.MAG}, {"U_HAT", d.UH}, {"DIFX", d.DIFX}, {"S_U", d.S_U}, {"UE", d.UE}, {"VN", d.VN},
        {"WT", d.WT}, {"U_N", d.U_N}, {"V_N", d.V_N}, {"W_N", d.W_N}, {"T_N", d.T_N}, {"NLX_NM1", d.NLX_NM1},
        {"NLY_NM1", d.NLY_NM1}, {"NLZ_NM1", d.NLZ_NM1}, {"ADV_NM1", d.ADV_NM1}};
    for (auto &e : t)
        if (!std::strcmp(e.n, name)) return e.a;
    return nullptr;
}

int bad3(fvm3_ctx *c, const char *m)
{
    if (c) c->err = m;
    return FVM_ERR_ARG;
}

}  // namespace
}  // namespace f3

extern "C" {

int fvm3_default_params(fvm3_params *p)
{
    if (!p) return FVM_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    p->ni = 241;   // comdat_param.f90:6-8
    p->nj = 201;
    p->nk = 121;
    p->re = 3900.0;
    p->pr = 0.71;
    p->dt = 1.0e-3;
    p->tin = 0.0;
    p->t_wall = 1.0;
    p->resimax = 1.0e-4;
    p->nswpp = 20;
    p->use_les = 1;
    p->les_zavg = 0;
    p->thermal = 1;
    p->res_every = 2;
    p->ref_a = 6.283185307;   // REF_A of comdat_param.f90:28
    p->precision = FVM_FP64;
    p->refine_sweeps = 8;
    p->device = 0;
    p->poisson_host_loop = 1;
    return FVM_OK;
}

int fvm3_create(const fvm3_params *p, fvm3_ctx **out)
{
    if (!out || !p) return FVM_ERR_ARG;
    *out = nullptr;
    if (p->ni < 6 || p->nj < 6 || p->nk < 6) return FVM_ERR_ARG;
    if ((p->nj - 1) % 2 || (p->nk - 1) % 2) return FVM_ERR_ARG;
    if (p->ni - 1 > 512 || p->nj - 1 > 512 || p->nk - 1 > 512) return FVM_ERR_ARG;
    if (!(p->dt > 0.0) || !(p->re > 0.0) || !(p->pr > 0.0) || p->nswpp < 1 || !(p->ref_a > 0.0)) return FVM_ERR_ARG;
    if (p->precision != FVM_FP64 && p->precision != FVM_MIXED) return FVM_ERR_ARG;
    if (p->precision == FVM_MIXED && p->refine_sweeps < 1) return FVM_ERR_ARG;
    if (p->tile_i_warps != 0 || p->tile_i_m != 0)
        if (!fvm::tile_supported(p->tile_i_warps, p->tile_i_m) || 32 * p->tile_i_warps * p->tile_i_m < p->ni - 1)
            return FVM_ERR_ARG;
    fvm3_ctx *c = new (std::nothrow) fvm3_ctx();
    if (!c) return FVM_ERR_NOMEM;
    c->p = *p;
    c->NI = p->ni;
    c->NJ = p->nj;
    c->NK = p->nk;
    c->n = (p->ni + 1) * (p->nj + 1) * (p->nk + 1);
    f3::D3 &d = c->d;
    d.NI = p->ni; d.NJ = p->nj; d.NK = p->nk; d.NI1 = p->ni + 1; d.NJ1 = p->nj + 1; d.n = c->n;
    d.re = p->re; d.pe = p->re * p->pr; d.dt = p->dt; d.rdt = 1.0 / p->dt; d.tin = p->tin; d.t_wall = p->t_wall;
    d.r2re_dt = (2.0 * d.re) / d.dt;
    d.r2pe_dt = (2.0 * d.pe) / d.dt;
    d.pi = 4.0 * std::atan(1.0); d.resimax = p->resimax; d.ref_a = p->ref_a;
    d.res_every = p->res_every < 1 ? 1 : p->res_every;
    d.nswpp = ((p->nswpp + d.res_every - 1) / d.res_every) * d.res_every;
    d.les_zavg = p->les_zavg; d.thermal = p->thermal;
    d.refine_sweeps = p->refine_sweeps < 1 ? 1 : p->refine_sweeps;
    if (p->precision == FVM_MIXED)
        d.nswpp = ((p->nswpp + d.refine_sweeps - 1) / d.refine_sweeps) * d.refine_sweeps;
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_pctl, sizeof(fvm::PCtl));
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_a);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_b);
    f3::Bump probe{nullptr};
    f3::carve(probe, c);
    if (e == cudaSuccess) e = cudaMalloc(&c->slab, probe.off + 256);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->slab, 0, probe.off + 256, c->stream);
    if (e != cudaSuccess) {
        fvm3_destroy(c);
        return FVM_ERR_NOMEM;
    }
    f3::Bump real{c->slab};
    f3::carve(real, c);
    *out = c;
    return FVM_OK;
}

int fvm3_destroy(fvm3_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->pgraph) cudaGraphExecDestroy(c->pgraph);
    if (c->slab) cudaFree(c->slab);
    if (c->post) cudaFree(c->post);
    if (c->h_pctl) cudaFreeHost(c->h_pctl);
    if (c->ev_a) cudaEventDestroy(c->ev_a);
    if (c->ev_b) cudaEventDestroy(c->ev_b);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FVM_OK;
}

const char *fvm3_last_error(const fvm3_ctx *c) { return c ? c->err.c_str() : "null context"; }

int fvm3_set_grid(fvm3_ctx *c, const double *xg, const double *yg, const double *zg)
{
    if (!c || !xg || !yg || !zg) return f3::bad3(c, "null grid pointer");
    const size_t bytes = sizeof(double) * c->n;
    F3CUDA(c, cudaMemcpyAsync(c->d.XG, xg, bytes, cudaMemcpyHostToDevice, c->stream));
    F3CUDA(c, cudaMemcpyAsync(c->d.YG, yg, bytes, cudaMemcpyHostToDevice, c->stream));
    F3CUDA(c, cudaMemcpyAsync(c->d.ZG, zg, bytes, cudaMemcpyHostToDevice, c->stream));
    int rc = f3::setup_grid(c);
    if (rc == FVM_OK) c->grid_set = true;
    return rc;
}

int fvm3_init(fvm3_ctx *c, const double *du, const double *dv, const double *dw)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) return f3::bad3(c, "fvm3_set_grid has not been called");
    const int n = c->n;
    std::vector<double> u(n, 1.0), z(n, 0.0), v(n, 0.0), w(n, 0.0);
    const int NI1 = c->NI + 1, NJ1 = c->NJ + 1;
    for (int k = 1; k <= c->NK - 1; k++)
        for (int j = 1; j <= c->NJ - 1; j++)
            for (int i = 1; i <= c->NI - 1; i++) {
                const int q = i + NI1 * (j + NJ1 * k);
                if (du) u[q] += du[q];
                if (dv) v[q] += dv[q];
                if (dw) w[q] += dw[q];
            }
    f3::D3 &d = c->d;
    const size_t bytes = sizeof(double) * n;
    F3CUDA(c, cudaMemcpyAsync(d.U, u.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    F3CUDA(c, cudaMemcpyAsync(d.V, v.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    F3CUDA(c, cudaMemcpyAsync(d.W, w.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    double *zero[] = {d.T, d.P, d.NLX, d.NLY, d.NLZ, d.ADV};
    for (double *a : zero) F3CUDA(c, cudaMemcpyAsync(a, z.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    c->rtime = 0.0;
    c->niter_time = 0;
    c->init_done = true;
    return FVM_OK;
}

int fvm3_step(fvm3_ctx *c, int nsteps, fvm3_coeffs *out)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->init_done) return f3::bad3(c, "fvm3_init has not been called");
    int status = FVM_OK;
    for (int s = 0; s < nsteps; s++) {
        F3RC(f3::step(c));
        F3RC(f3::read_coeffs(c, out));
        if (c->last.resid > c->p.resimax) status = FVM_ERR_NOCONV;
    }
    return status;
}

int fvm3_get_array(fvm3_ctx *c, const char *name, double *out)
{
    if (!c || !name || !out) return f3::bad3(c, "null argument");
    double *a = f3::array_by_name(c, name);
    if (!a) return f3::bad3(c, "unknown array name");
    F3CUDA(c, cudaMemcpyAsync(out, a, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

int fvm3_set_array(fvm3_ctx *c, const char *name, const double *in)
{
    if (!c || !name || !in) return f3::bad3(c, "null argument");
    double *a = f3::array_by_name(c, name);
    if (!a) return f3::bad3(c, "unknown array name");
    F3CUDA(c, cudaMemcpyAsync(a, in, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->stream));
    if (c->d.dfl && a >= c->shadow_lo && a < c->shadow_hi) F3RC(f3::refresh(c, {a}));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    c->init_done = true;
    return FVM_OK;
}

int fvm3_upload_state(fvm3_ctx *c, const double *u, const double *v, const double *w, const double *p,
                      const double *t, const double *nlx, const double *nly, const double *nlz, const double *adv)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) return f3::bad3(c, "fvm3_set_grid has not been called");
    const size_t bytes = sizeof(double) * c->n;
    f3::D3 &d = c->d;
    const double *src[] = {u, v, w, p, t, nlx, nly, nlz, adv};
    double *dst[] = {d.U, d.V, d.W, d.P, d.T, d.NLX, d.NLY, d.NLZ, d.ADV};
    std::vector<double *> shadowed;
    for (int k = 0; k < 9; k++) {
        if (!src[k]) continue;
        F3CUDA(c, cudaMemcpyAsync(dst[k], src[k], bytes, cudaMemcpyHostToDevice, c->stream));
        if (c->d.dfl && dst[k] >= c->shadow_lo && dst[k] < c->shadow_hi) shadowed.push_back(dst[k]);
    }
    if (!shadowed.empty()) F3RC(f3::refresh(c, shadowed));   // double-float shadows (mixed path)
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    c->init_done = true;
    return FVM_OK;
}

int fvm3_download_state(fvm3_ctx *c, double *u, double *v, double *w, double *p, double *t, double *nlx,
                        double *nly, double *nlz, double *adv)
{
    if (!c) return FVM_ERR_ARG;
    const size_t bytes = sizeof(double) * c->n;
    f3::D3 &d = c->d;
    double *dst[] = {u, v, w, p, t, nlx, nly, nlz, adv};
    const double *src[] = {d.U, d.V, d.W, d.P, d.T, d.NLX, d.NLY, d.NLZ, d.ADV};
    for (int k = 0; k < 9; k++)
        if (dst[k]) F3CUDA(c, cudaMemcpyAsync(dst[k], src[k], bytes, cudaMemcpyDeviceToHost, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

int fvm3_sgs(fvm3_ctx *c, fvm3_coeffs *out)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->init_done) return f3::bad3(c, "fvm3_init has not been called");
    // the model on the current state: the step-n copies and far-field values first
    f3::D3 &d = c->d;
    f3::k3_begin<<<f3::g_lin(c), 256, 0, c->stream>>>(d);
    f3::k3_farfield<<<dim3((c->NJ + 127) / 128, c->NK - 1), 128, 0, c->stream>>>(d);
    F3RC(f3::refresh(c, {d.U_N, d.V_N, d.W_N, d.T_N}));
    F3CUDA(c, cudaMemsetAsync(d.NLX, 0, sizeof(double) * c->n, c->stream));
    F3CUDA(c, cudaMemsetAsync(d.NLY, 0, sizeof(double) * c->n, c->stream));
    F3CUDA(c, cudaMemsetAsync(d.NLZ, 0, sizeof(double) * c->n, c->stream));
    F3CUDA(c, cudaMemsetAsync(d.ADV, 0, sizeof(double) * c->n, c->stream));
    F3RC(f3::sgs(c));
    double s[2];
    F3CUDA(c, cudaMemcpyAsync(s, d.scal, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->cs2 = s[0];
        out->ct2 = s[1];
    }
    return FVM_OK;
}

// ---------------------------------------------------------------------------------
// Per-routine call points (fvm3_step runs them in this order)
// ---------------------------------------------------------------------------------
#define F3READY(c)                                                        \
    do {                                                                  \
        if (!(c)) return FVM_ERR_ARG;                                     \
        if (!(c)->init_done) return f3::bad3((c), "fvm3_init has not been called"); \
    } while (0)

int fvm3_begin_step(fvm3_ctx *c) { F3READY(c); return f3::begin_step(c); }
int fvm3_contra_vel(fvm3_ctx *c) { F3READY(c); return f3::contra_vel(c, 0); }
int fvm3_nl(fvm3_ctx *c) { F3READY(c); return f3::nl_all(c); }
int fvm3_stress_tensor(fvm3_ctx *c)
{
    F3READY(c);
    return c->p.use_les ? f3::sgs(c) : FVM_OK;
}
int fvm3_dif(fvm3_ctx *c) { F3READY(c); return f3::dif_all(c); }
int fvm3_p_source(fvm3_ctx *c) { F3READY(c); return f3::p_source(c); }
int fvm3_iter_u(fvm3_ctx *c, int component)
{
    F3READY(c);
    if (component < 0 || component > 2) return f3::bad3(c, "component must be 0 (U), 1 (V) or 2 (W)");
    return f3::iter_u(c, component);
}
int fvm3_remove_grad(fvm3_ctx *c) { F3READY(c); return f3::remove_grad(c); }
int fvm3_iter_p(fvm3_ctx *c, double *resid, int *sweeps)
{
    F3READY(c);
    F3RC(f3::iter_p(c));
    F3CUDA(c, cudaMemcpyAsync(c->h_pctl, c->d.pctl, sizeof(fvm::PCtl), cudaMemcpyDeviceToHost, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    if (resid) *resid = c->h_pctl->resip;
    if (sweeps) *sweeps = c->h_pctl->niter;
    if (!std::isfinite(c->h_pctl->resip)) {
        c->err = "non-finite Poisson residual";
        return FVM_ERR_NAN;
    }
    return c->h_pctl->capped ? FVM_ERR_NOCONV : FVM_OK;
}
int fvm3_correct(fvm3_ctx *c) { F3READY(c); return f3::correct(c); }
int fvm3_iter_t(fvm3_ctx *c) { F3READY(c); return f3::iter_t(c); }
int fvm3_calccoef(fvm3_ctx *c, fvm3_coeffs *out)
{
    F3READY(c);
    F3RC(f3::calccoef(c));
    return f3::read_coeffs(c, out);
}

int fvm3_test_filter(fvm3_ctx *c, const double *in, double *out)
{
    if (!c || !in || !out) return f3::bad3(c, "null argument");
    if (!c->grid_set) return f3::bad3(c, "fvm3_set_grid has not been called");
    f3::D3 &d = c->d;
    const size_t bytes = sizeof(double) * c->n;
    // LM and MM are scratch of the SGS model between its own kernels
    F3CUDA(c, cudaMemcpyAsync(d.LM, in, bytes, cudaMemcpyHostToDevice, c->stream));
    F3CUDA(c, cudaMemcpyAsync(d.MM, out, bytes, cudaMemcpyHostToDevice, c->stream));
    f3::k3_filter<double><<<f3::g_int(c), f3::B_INT, 0, c->stream>>>(d, d.LM, d.MM);
    F3CHECK(c);
    F3CUDA(c, cudaMemcpyAsync(out, d.MM, bytes, cudaMemcpyDeviceToHost, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

// ---------------------------------------------------------------------------------
// Post-processing (post_process.f90:8-285)
// ---------------------------------------------------------------------------------
int fvm3_post_begin(fvm3_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) return f3::bad3(c, "fvm3_set_grid has not been called");
    const size_t bytes = sizeof(double) * 17 * size_t(c->n);
    if (!c->post) F3CUDA(c, cudaMalloc(&c->post, bytes));
    F3CUDA(c, cudaMemsetAsync(c->post, 0, bytes, c->stream));
    F3CUDA(c, cudaStreamSynchronize(c->stream));
    c->niter_pos = 0;
    c->ipost = 1;
    return FVM_OK;
}

int fvm3_post_end(fvm3_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    c->ipost = 0;
    return FVM_OK;
}

int fvm3_post_steps(fvm3_ctx *c, int *steps)
{
    if (!c || !steps) return FVM_ERR_ARG;
    *steps = c->niter_pos;
    return FVM_OK;
}

namespace {
int down(fvm3_ctx *c, const double *dev, std::vector<double> &h)
{
    h.resize(c->n);
    F3CUDA(c, cudaMemcpyAsync(h.data(), dev, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
    return FVM_OK;
}
}  // namespace

int fvm3_post_get(fvm3_ctx *c, const char *name, double *out)
{
    if (!c || !name || !out) return f3::bad3(c, "null argument");
    if (!c->post || c->niter_pos < 1) return f3::bad3(c, "no post-processing steps have been averaged");
    const int n = c->n;
    const double N = (double)c->niter_pos;
    const double *ps = c->post;
    auto sum = [&](int q, std::vector<double> &h) { return down(c, ps + size_t(q) * n, h); };
    auto sync = [&]() -> int { F3CUDA(c, cudaStreamSynchronize(c->stream)); return FVM_OK; };
    static const char *avg[] = {"U_AVG", "V_AVG", "W_AVG", "P_AVG", "T_AVG"};
    static const char *rs[] = {"UU", "UV", "UW", "VV", "VW", "WW"};
    static const char *rms[] = {"U_RMS", "V_RMS", "W_RMS"};
    static const int ra[] = {0, 0, 0, 1, 1, 2}, rb[] = {0, 1, 2, 1, 2, 2}, rq[] = {5, 8, 10};
    std::vector<double> a, b, m, sg;
    for (int q = 0; q < 5; q++)
        if (!std::strcmp(name, avg[q])) {   // post_process.f90:61-65
            F3RC(sum(q, a));
            F3RC(sync());
            for (int e = 0; e < n; e++) out[e] = a[e] / N;
            return FVM_OK;
        }
    for (int q = 0; q < 6; q++)
        if (!std::strcmp(name, rs[q])) {   // post_process.f90:156-167, 207-212
            F3RC(sum(ra[q], a));
            F3RC(sum(rb[q], b));
            F3RC(sum(5 + q, m));
            F3RC(sum(11 + q, sg));
            F3RC(sync());
            for (int e = 0; e < n; e++) out[e] = (m[e] / N - (a[e] / N) * (b[e] / N)) + sg[e] / N;
            return FVM_OK;
        }
    for (int q = 0; q < 3; q++)
        if (!std::strcmp(name, rms[q])) {   // post_process.f90:164-166
            F3RC(sum(rq[q], m));
            F3RC(sync());
            for (int e = 0; e < n; e++) out[e] = std::sqrt(m[e] / N);
            return FVM_OK;
        }
    const int which = !std::strcmp(name, "CF_WALL") ? 0 : (!std::strcmp(name, "CP_WALL") ? 1 : (!std::strcmp(name, "NU_WALL") ? 2 : -1));
    if (which < 0) return f3::bad3(c, "unknown post-processing array name");
    // wall statistics of the averaged fields (post_process.f90:67-116, 252-255)
    const f3::D3 &d = c->d;
    std::vector<double> f[5], XG, YG, ZG, X, Y, Z, A1, A2;
    for (int q = 0; q < 5; q++) F3RC(sum(q, f[q]));
    F3RC(down(c, d.XG, XG)); F3RC(down(c, d.YG, YG)); F3RC(down(c, d.ZG, ZG));
    F3RC(down(c, d.X, X)); F3RC(down(c, d.Y, Y)); F3RC(down(c, d.Z, Z));
    F3RC(down(c, d.AREA1, A1)); F3RC(down(c, d.AREA2, A2));
    F3RC(sync());
    for (int q = 0; q < 5; q++)
        for (int e = 0; e < n; e++) f[q][e] = f[q][e] / N;
    const int NI1 = c->NI + 1, NJ1 = c->NJ + 1;
    auto id = [&](int i, int j, int k) { return i + NI1 * (j + NJ1 * k); };
    for (int e = 0; e < NJ1 * (c->NK + 1); e++) out[e] = 0.0;
    for (int k = 1; k <= c->NK - 1; k++)
        for (int j = 1; j <= c->NJ - 1; j++) {
            const int i = 1, cc = id(i, j, k);
            double sh = 0.0, nus = 0.0;
            for (int tri = 0; tri < 2; tri++) {
                int p, q, r;
                if (tri == 0) { p = id(i, j, k); q = id(i, j + 1, k); r = id(i, j, k + 1); }
                else { p = id(i, j + 1, k + 1); q = id(i, j, k + 1); r = id(i, j, k); }
                const double A = (YG[p] * (ZG[q] - ZG[r]) + YG[q] * (ZG[r] - ZG[p])) + YG[r] * (ZG[p] - ZG[q]);
                const double B = (ZG[p] * (XG[q] - XG[r]) + ZG[q] * (XG[r] - XG[p])) + ZG[r] * (XG[p] - XG[q]);
                const double C = (XG[p] * (YG[q] - YG[r]) + XG[q] * (YG[r] - YG[p])) + XG[r] * (YG[p] - YG[q]);
                double D = (XG[p] * (YG[q] * ZG[r] - YG[r] * ZG[q]) + XG[q] * (YG[r] * ZG[p] - YG[p] * ZG[r])) +
                           XG[r] * (YG[p] * ZG[q] - YG[q] * ZG[p]);
                D = -1.0 * D;
                const double dum = std::sqrt((A * A + B * B) + C * C);
                const double dn = std::fabs(((A * X[cc] + B * Y[cc]) + C * Z[cc]) + D) / dum;
                const double u = f[0][cc], v = f[1][cc], w = f[2][cc];
                const double e1 = (v * C) / dum - (w * B) / dum, e2 = (u * C) / dum - (w * A) / dum,
                             e3 = (u * B) / dum - (v * A) / dum;
                const double dudn = std::sqrt((e1 * e1 + e2 * e2) + e3 * e3) / dn;
                const double dtdn = (f[4][cc] - c->p.t_wall) / dn;
                const double ar = tri == 0 ? A1[cc] : A2[cc], tot = A1[cc] + A2[cc];
                sh = sh + (dudn * ar) / tot;
                nus = nus + (dtdn * ar) / tot;
            }
            const std::vector<double> &P = f[3];
            const double pg = 0.125 * (((((((P[id(i, j, k)] + P[id(i, j - 1, k)]) + P[id(i - 1, j, k)]) +
                                          P[id(i - 1, j - 1, k)]) + P[id(i, j, k + 1)]) + P[id(i, j - 1, k + 1)]) +
                                        P[id(i - 1, j, k + 1)]) + P[id(i - 1, j - 1, k + 1)]);
            const double v3[3] = {(2.0 / std::sqrt(c->p.re)) * sh, 2.0 * pg, -nus};
            out[j + NJ1 * k] = v3[which];
        }
    return FVM_OK;
}

int fvm3_time_sweeps(fvm3_ctx *c, int sweeps, double *ms_per_sweep)
{
    if (!c || sweeps < 1 || !ms_per_sweep) return FVM_ERR_ARG;
    f3::D3 &d = c->d;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    // the sweeps of the loop body on a scratch copy of P (SU as left by the last step)
    F3CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = FVM_OK;
    const bool mixed = c->p.precision == FVM_MIXED;
    for (int s = 0; s < sweeps && rc == FVM_OK; s++) {
        if (mixed) {
            rc = f3::line32(c, 0, 0, 0);
            if (rc == FVM_OK) rc = f3::line32(c, 1, 0, 0);
        } else {
            rc = f3::line(c, 6, d.SU, d.DIVDT, 0);
            if (rc == FVM_OK) rc = f3::line(c, 6, d.SU, d.DIVDT, 1);
        }
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : FVM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return FVM_ERR_CUDA;
    F3CUDA(c, cudaGraphLaunch(ge, c->stream));
    F3CUDA(c, cudaEventRecord(c->ev_a, c->stream));
    F3CUDA(c, cudaGraphLaunch(ge, c->stream));
    F3CUDA(c, cudaEventRecord(c->ev_b, c->stream));
    F3CUDA(c, cudaEventSynchronize(c->ev_b));
    float ms = 0.f;
    F3CUDA(c, cudaEventElapsedTime(&ms, c->ev_a, c->ev_b));
    cudaGraphExecDestroy(ge);
    *ms_per_sweep = ms / sweeps;
    return FVM_OK;
}

int fvm3_get_stream(fvm3_ctx *c, void **stream)
{
    if (!c || !stream) return FVM_ERR_ARG;
    *stream = c->stream;
    return FVM_OK;
}

}  // extern "C"
