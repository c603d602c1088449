// fvm_internal.cuh -- device data layout, context and shared device helpers of the
// GB300 cylinder time step.  All arrays live in one device slab; every field array
// is the reference's Fortran (0:NI,0:NJ) array, element (i,j) at i + (NI+1)*j.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <type_traits>
#include <vector>

#include "../../include/fvm.h"

namespace fvm {

constexpr int WARP = 32;
constexpr int RES_CELLS = 2;   // cells per thread of the mixed and adjoint Poisson residual kernels
// cells per thread of the FP64 path's residual (k_pres64): eight amortise the block
// reduction over more cells and leave room for the overlapping sweep launches (FP64
// step 39.7 -> 35.7 ms on 512 x 384; two, for the mixed path's k_mres, measured best)
constexpr int RES64_CELLS = 8;
// Tile of the mixed path's residual kernel k_mres: 32 radial x 8 circumferential
// cells per 256-thread block, the pressure of the tile and its halo split into
// double-float once in shared memory.
constexpr int MRES_TI = 32, MRES_TJ = 8;

// One set of constant tridiagonal factors for a family of lines (one line per
// radial row j, or per circumferential column i), solved by groups of NW warps
// (TG = 32*NW threads).  Factors are stored chunk-interleaved: element
// e = t*M + k of line L sits at L*TG*M + k*TG + t, so every group-wide load of one
// k is coalesced.  Padding elements (e >= n) have zero factors and never influence
// real elements.
struct LineSys {
    int lines = 0;     // number of lines
    int n = 0;         // unknowns per line
    int NW = 1;        // warps per line group
    int M = 0;         // elements per thread (ceil(n/(32*NW)))
    int cyclic = 0;    // 1: periodic line solved by Sherman-Morrison
    double *invD = nullptr, *fa = nullptr, *fb = nullptr, *z = nullptr;  // FP64 factors
    float *invDf = nullptr, *faf = nullptr, *fbf = nullptr, *zf = nullptr; // FP32 copies
    double *cv = nullptr, *sinv = nullptr;   // cyclic: a_1/gamma and 1/(1+v.z) per line
    float *cvf = nullptr, *sinvf = nullptr;
};

// Five-point coefficient set of one AF factor or of the Poisson operator, with the
// boundary-condition folding already applied (constant for the run).
struct Coef {
    double *AP = nullptr, *AE = nullptr, *AW = nullptr, *AN = nullptr, *AS = nullptr;
    float *ANf = nullptr, *ASf = nullptr, *AEf = nullptr, *AWf = nullptr;
    double *awall = nullptr;   // raw AW(1,j) before folding (per j)
    double *afar = nullptr;    // raw AE(NI-1,j) before folding (per j)
};

// Device control block of the Poisson iteration.
struct PCtl {
    int niter;          // sweeps done in the current ITER_P
    int done;           // 1 once converged or capped
    int capped;         // 1 if stopped at the cap above tolerance
    int fault;          // 1 if a bounded wait of the resident sweep kernel ran out
    double resip;       // last scaled residual
    unsigned int ticket;
    unsigned int xbase;   // resident path: the blocks' sweep count (XCNT) when the step's Poisson loop began
    double pad3;
};

// Batch-wide control block of a batched launch (device memory).
struct BatchCtl {
    int remaining;      // cases whose Poisson iteration of this step is still running
    int ncases;
    int step;           // steps recorded in the current batch call
    int bodies;         // Poisson loop bodies run in this step
    int max_bodies;     // bound on bodies per step (every case reaches its cap before)
    int overrun;        // set if the bound ended the loop
};

// Everything a kernel needs, passed by value.
struct Dev {
    int NI, NJ, NI1, n;
    double re, pe, dt, rdt, vel_rot, uin, vin, tin, t_wall, pi, resimax;
    int nswpp;          // sweep cap, rounded up to a multiple of the residual interval
    int res_every;      // FP64: residual interval (even, >= 2)
    int iter_t_bug;
    int dd_pos;         // 1: cell (i,j) takes the cross term of cell (i-1,j-1) in DIF / ITER_P
    int refine_sweeps;  // MIXED: FP32 sweeps per FP64 refinement
    int adi_refine;     // MIXED: defect-correction passes of a predictor line
    int nblk_res;       // blocks of this case in the residual kernels (RES_CELLS per thread)
    int nblk_res64;     // blocks of this case in the FP64 path's residual (RES64_CELLS per thread)
    int nblk_mres;      // blocks of this case in the mixed path's residual (MRES_TI x MRES_TJ tiles)
    int case_id;        // position in a batch
    BatchCtl *bctl;     // batch control (nullptr in a single-context launch)
    fvm_coeffs *bhist;  // batch: coefficient records [step * ncases + case]
    double *btime;      // batch: the case's simulated time, advanced on the device
    // geometry
    double *XG, *YG, *X, *Y, *XIX, *XIY, *ETX, *ETY, *DJAC, *Q11, *Q12, *Q22;
    double *DE, *DW, *DN, *DS, *THETA, *AREA;
    double *JQ12;          // DJAC*Q12
    // Poisson cross term DD = CNE P(i+1,j+1) + CSE P(i+1,j-1) + CNW P(i-1,j+1) + CSW P(i-1,j-1),
    // the four diagonal weights of dif_diagonal.f90:13-23 gathered per cell (interior)
    double *CNE, *CSE, *CNW, *CSW;
    double *JXE, *JYE;     // (DJAC*XIX)*ETX and (DJAC*XIY)*ETY
    double *RJDT;          // (2*RE)*DJAC/DT  and for Pe:
    double *PJDT;          // (2*PE)*DJAC/DT
    double *UFW, *VFW, *TFW;  // wall boundary values per j (constant)
    double *BLOW, *WB;        // wall blowing speed per j (control) and its face-flux weight
    double *FFU, *FFV, *FFT;  // far-field boundary values per j (per step)
    // state
    double *U, *V, *P, *T, *U_N, *V_N, *T_N;
    double *P2;            // second pressure buffer of the double-buffered FP64 zebra sweep
    double *NLX, *NLY, *ADV, *NLX_NM1, *NLY_NM1, *ADV_NM1, *DIFX, *DIFY, *DIFT, *S_U, *S_V;
    double *UE, *UW, *VN, *VS, *DIVDT;
    double *SU, *SUV, *SUT, *DD;   // per-field right-hand sides (U uses SU)
    // mixed-precision scratch
    float *RF, *DF;                // FP32 residual right-hand side and correction
    // AE, AW, AN, AS, AP of the pressure equation and CNE, CSE, CNW, CSW, each split
    // into double-float (hi, lo): nine planes of n cells for the mixed residual
    float2 *PCD;
    // line-resident sweeps: boundary-line exchange words (value bits | tag << 32),
    // [slot 0/1][line][element], and each block's count of completed sweeps
    unsigned long long *XW;
    unsigned int *XCNT;
    double *W64;                   // FP64 scratch line values (defect correction)
    // reductions
    PCtl *pctl;
    double *partial;               // per-block partial sums (2 per block)
    double *coefrow;               // per-j CALCCOEF contributions (6 per j)
    unsigned long long *cflbits;
    double *scal;                  // small scalars: [0]=sum_area
    // line systems and coefficients
    Coef cP, cUX, cUY, cTX, cTY;
    LineSys sP, sUX, sUY, sTX, sTY;
};

// Source of a kernel's Dev: one context (the Dev itself, passed by value) or a
// batch (a table of Dev in device memory, one per case, case = blockIdx.z).
struct DevTable {
    const Dev *devs;
};
__device__ __forceinline__ const Dev &dev_of(const Dev &d) { return d; }
__device__ __forceinline__ const Dev &dev_of(const DevTable &t) { return t.devs[blockIdx.z]; }

}  // namespace fvm

struct fvm_adj;   // adjoint storage (fvm_adjoint.cu), created on first use

namespace fvm {
// Post-processing state of CALCCOEF / POST_PROCESS (comdat_shared.f90:149-160):
// the scalars on the host, the field sums on the device.
struct PostState {
    int ipost = 0, toggle = 0, niter_pos = 0;
    double cl1 = 0.0, st = 0.0, cl_amp = 0.0, time1 = 0.0, time2 = 0.0;
    double nu_ta = 0.0, cd_ta = 0.0, cl_ta = 0.0, st_ta = 0.0, cpb_ta = 0.0, cl_amp_ta = 0.0;
    double rms_cd = 0.0, rms_cl = 0.0;
    fvm_post rec{};
    double *arr = nullptr;   // device: VOR, U_TA, V_TA, P_TA, T_TA, VOR_TA (n each)
};
}  // namespace fvm

struct fvm_ctx {
    fvm_params p{};
    int NI = 0, NJ = 0, NI1 = 0, n = 0;
    cudaStream_t stream = nullptr;
    fvm::Dev d{};
    char *slab = nullptr;
    size_t slab_bytes = 0;
    std::string err;
    bool grid_set = false, init_done = false;
    double rtime = 0.0;
    int niter_time = 0;
    fvm_coeffs last{};
    std::vector<fvm_coeffs> hist;
    fvm::PCtl *h_pctl = nullptr;     // pinned mirror
    // Poisson graph: a batch of sweeps replayed until converged
    cudaGraphExec_t pgraph = nullptr;
    int pgraph_batch = 0;
    int nblk_res = 0;      // blocks of the residual kernels
    int nblk_res64 = 0;    // blocks of the FP64 path's residual kernel
    int nblk_mres = 0;     // blocks of the mixed path's residual kernel
    // instrumentation
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;   // span around the first sweep group of a replay
    int pgraph_kernels = 0;                       // kernel nodes in the Poisson graph
    int span_launches = 0;                        // sweep kernels inside the span
    bool capturing = false;
    fvm_timing tm{};
    fvm_adj *adj = nullptr;
    // line-resident Poisson sweeps (mixed path): lines per block (0: per-colour
    // launches), blocks, and whether the launch carries the cooperative attribute
    int res_lines = 0, res_blocks = 0;
    int res_depth = 1;   // sweeps per boundary-line exchange (1, or 2 with 4 lines per block)
    bool res_coop = false;
    fvm::PostState post;
    int post_suspend = 0;   // recomputation passes of the adjoint: no post-processing
};

// Count one kernel launch of the context (into the graph being captured, if any).
#define KCOUNT(c)                                             \
    do {                                                      \
        if ((c)->capturing) (c)->pgraph_kernels++;            \
        else (c)->tm.kernel_launches++;                       \
    } while (0)

// ---------------------------------------------------------------------------------
// Host helpers shared by the translation units
// ---------------------------------------------------------------------------------
#define FVM_CUDA(ctx, call)                                                                  \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
            return FVM_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

#define FVM_LAUNCH_CHECK(ctx)                                                                \
    do {                                                                                     \
        cudaError_t e_ = cudaGetLastError();                                                 \
        if (e_ != cudaSuccess) {                                                             \
            (ctx)->err = std::string("kernel launch: ") + cudaGetErrorString(e_);            \
            return FVM_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

namespace fvm {
// Where the launches of a step go: one context, or a batch of contexts advanced
// together (grid z = case; x/y extents are the maxima over the cases, surplus
// blocks of smaller cases return at once).  The cases of a batch share the line
// tiles and the run options that shape the launch sequence.
struct Tgt {
    fvm_ctx *c = nullptr;        // error text and launch counters
    cudaStream_t st = nullptr;   // stream the launches go to
    const Dev *one = nullptr;    // single context: its device view (passed by value)
    DevTable tab{nullptr};       // batch: device table of the cases' views
    int nz = 1;                  // cases
    int NI = 0, NJ = 0, n = 0, nblk_res = 0, nblk_res64 = 0, nblk_mres = 0;   // launch extents
    LineSys tr{}, tt{};          // tiles (NW, M) of the radial and circumferential line families
    int mixed = 0, thermal = 1, iter_t_bug = 1, refine_sweeps = 1, res_every = 2;
};

template <class F>
inline void with_src(const Tgt &t, F &&f)
{
    if (t.tab.devs) f(t.tab);
    else f(*t.one);
}

Tgt tgt_of(fvm_ctx *c);
int setup_allocate(fvm_ctx *c);
void radial_tile(const fvm_ctx *c, int &nw, int &m);
int setup_factors(fvm_ctx *c);
void split_pcoef(fvm_ctx *c);   // double-float planes of the pressure coefficients (d.PCD)
int setup_controls(fvm_ctx *c, double omega, const double *blow);
int setup_grid(fvm_ctx *c);
int setup_init(fvm_ctx *c, const double *du, const double *dv);
int run_begin_step(fvm_ctx *c);
int run_contra_vel(fvm_ctx *c);
int run_nl(fvm_ctx *c, int field);
int run_dif(fvm_ctx *c, int field);
int run_p_source(fvm_ctx *c);
int run_iter_u(fvm_ctx *c, int field);
int run_remove_grad(fvm_ctx *c);
int run_iter_p(fvm_ctx *c, double *resid, int *sweeps);
int run_correct(fvm_ctx *c);
int run_iter_t(fvm_ctx *c);
int run_calccoef(fvm_ctx *c, fvm_coeffs *out);
// post-processing block of CALCCOEF for a step whose record is co; cl_prev is
// the previous step's lift (CL_NM1, calccoef.f90:109)
int post_after_calccoef(fvm_ctx *c, double cl_prev, const fvm_coeffs &co);
void post_free(fvm_ctx *c);
double *post_array(fvm_ctx *c, const char *name);
int run_step(fvm_ctx *c, int nsteps, fvm_coeffs *out);
double *array_by_name(fvm_ctx *c, const char *name);
int run_time_sweeps(fvm_ctx *c, int sweeps, double *ms_per_launch, long long *launches);
int run_resident_wait_test(fvm_ctx *c, int max_polls);
// launch sequences shared by single contexts and batches (fvm_step.cu)
int step_before_poisson(const Tgt &t);
int poisson_bodies(const Tgt &t, cudaGraphConditionalHandle cond, int has_cond, int groups);
int step_after_poisson(const Tgt &t, double rtime, fvm_coeffs *dout);
int sweep_pairs(const Tgt &t, int sweeps);
int launch_batch_tick(const Tgt &t, BatchCtl *b);
// discrete adjoint (fvm_adjoint.cu)
int run_adjoint(fvm_ctx *c, int window, int ckpt, double *J, double *dJ_domega, double *dJ_dblow);
int run_adjoint_vjp(fvm_ctx *c, double *const *lam, double *dctrl);
void adj_destroy(fvm_ctx *c);
int theta_pairs(const Tgt &t, int field, int sweeps);
int predictor_sweeps(const Tgt &t, int field);
// mixed precision (fvm_mixed.cu)
int mixed_poisson_body(const Tgt &t, cudaGraphConditionalHandle cond, int has_cond);
int mixed_sweep_pair(const Tgt &t, int apply);
int mixed_predictor_radial(const Tgt &t, int field, int colour, int refresh);
int mixed_predictor_theta(const Tgt &t, int field, int colour, int ghosts);
// line-resident FP32 sweeps (fvm_resident.cu).  The correction system a launch
// solves: line factors (in the layout of the context's radial tile) and couplings,
// the FP32 right-hand side and correction, the FP64 field the correction is added
// to (bcp = 1: with the BCP ghost refresh of each updated row, the forward pressure;
// 0: interior only) and the iteration's control block.
struct ResSys {
    const float *invDf, *faf, *fbf;
    const float *ANf, *ASf;
    const float *RF;
    float *DF;
    double *X;
    PCtl *pctl;
    int bcp;
    // 1: the launch first sums the block partials the forward residual kernel left
    // and takes the loop's convergence decision (forward Poisson loop only)
    int decide;
};
int resident_setup(fvm_ctx *c);
// the same launch on another system (the adjoint's transposed Poisson equation)
int resident_sweeps_on(fvm_ctx *c, const ResSys &sys, int sweeps, int apply, int check_done);
int resident_sweeps(const Tgt &t, int sweeps, int apply, int max_polls, unsigned tag_skew,
                    cudaGraphConditionalHandle cond, int has_cond, int check_done, int decide = 0);
int resident_reset(fvm_ctx *c);
}  // namespace fvm

// ---------------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------------
#define IDX(i, j) ((i) + d.NI1 * (j))

namespace fvm {

// Ghost cells derived from interior cell (i,j) after it takes value val: the wall
// ghost (i=1), the far-field ghost (i=NI-1) of the Dirichlet-by-ghost condition
// phi_ghost = -phi + 2 phi_boundary (bcu.f90:18,38), and the branch-cut copies
// (bcu.f90:44-51), including the corner cells the reference fills by the copy.
__device__ __forceinline__ void ghost_dirichlet(const Dev &d, double *phi, int i, int j, double val,
                                                const double *wallF, const double *farF)
{
    const int NI = d.NI, NJ = d.NJ;
    if (i == 1) {
        double g = (-val) + 2.0 * wallF[j];
        phi[IDX(0, j)] = g;
        if (j == 1) phi[IDX(0, NJ)] = g;
        if (j == NJ - 1) phi[IDX(0, 0)] = g;
    }
    if (i == NI - 1) {
        double g = (-val) + 2.0 * farF[j];
        phi[IDX(NI, j)] = g;
        if (j == 1) phi[IDX(NI, NJ)] = g;
        if (j == NJ - 1) phi[IDX(NI, 0)] = g;
    }
    if (j == 1) phi[IDX(i, NJ)] = val;
    if (j == NJ - 1) phi[IDX(i, 0)] = val;
}

__device__ __forceinline__ int jwrap(const Dev &d, int j)
{
    return j == 0 ? d.NJ - 1 : (j == d.NJ ? 1 : j);
}

template <typename T>
__device__ __forceinline__ T shfl_up(T v, int s) { return __shfl_up_sync(0xffffffffu, v, s); }
template <typename T>
__device__ __forceinline__ T shfl_down(T v, int s) { return __shfl_down_sync(0xffffffffu, v, s); }
template <typename T>
__device__ __forceinline__ T shfl_idx(T v, int s) { return __shfl_sync(0xffffffffu, v, s); }

// ---------------------------------------------------------------------------------
// Line solves by a group of NW warps (TG = 32*NW threads).  Thread t of the group
// owns the chunk e = t*M .. t*M+M-1 of the line; the constant factors are stored
// chunk-interleaved (element e = t*M + k at line_base + k*TG + t) so that every
// factor load is coalesced.  Field arrays are read and written in the interleaved
// ownership e = k*TG + t (coalesced along a Fortran row) and moved between the two
// ownerships through shared memory.
// ---------------------------------------------------------------------------------
template <int NW>
__device__ __forceinline__ void gsync()
{
    if (NW > 1) __syncthreads();
    else __syncwarp();
}

// Barrier of one line group: the whole block (the group is the block, or every
// group of the block runs the same barrier sequence) ...
template <int NW>
struct BlockSync {
    __device__ __forceinline__ void operator()() const { gsync<NW>(); }
};
// ... or the group's own named barrier (id >= 1, the group's 32*NW threads), so that
// groups of one block synchronise independently.
template <int NW>
struct NamedSync {
    int id;
    __device__ __forceinline__ void operator()() const
    {
        if (NW > 1) asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(WARP * NW) : "memory");
        else __syncwarp();
    }
};

__device__ __forceinline__ int spad(int e) { return e + (e >> 5); }

// Rounded operations whose order the compiler cannot change.  An expression with
// two products and a sum may be contracted either way; these fix the form, so that
// every kernel computing the same quantity gives the same bits.
// (other arithmetic types, e.g. double-float pairs: their own operators, a*b then + c)
template <typename T>
__device__ __forceinline__ T fma_rn(T a, T b, T c) { return a * b + c; }
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b) { return a * b; }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// Right-hand side of a line of the FP32 Poisson correction sweep:
// (AN x(j+1) + AS x(j-1)) + r, in one fixed rounding order.
__device__ __forceinline__ float pois32_rhs(float an, float xn, float as, float xs, float r)
{
    return add_rn(fma_rn(an, xn, mul_rn(as, xs)), r);
}

template <typename T, int M, int NW, class Sync = BlockSync<NW>>
__device__ __forceinline__ void to_chunks(T (&v)[M], T *sm, int t, Sync sync = Sync())
{
    constexpr int TG = WARP * NW;
#pragma unroll
    for (int k = 0; k < M; k++) sm[spad(k * TG + t)] = v[k];
    sync();
#pragma unroll
    for (int k = 0; k < M; k++) v[k] = sm[spad(t * M + k)];
    sync();
}

template <typename T, int M, int NW, class Sync = BlockSync<NW>>
__device__ __forceinline__ void to_interleaved(T (&v)[M], T *sm, int t, Sync sync = Sync())
{
    constexpr int TG = WARP * NW;
#pragma unroll
    for (int k = 0; k < M; k++) sm[spad(t * M + k)] = v[k];
    sync();
#pragma unroll
    for (int k = 0; k < M; k++) v[k] = sm[spad(k * TG + t)];
    sync();
}

// Apply the precomputed LU factors of one line to the right-hand side held in
// chunk ownership, in place:
//   forward:  y_e = invD_e r_e + fa_e y_{e-1}
//   backward: x_e = y_e + fb_e x_{e+1}
// Each first-order recurrence runs sequentially inside a chunk, the chunks are
// combined by a Kogge-Stone scan of affine maps across the warp and by a short
// fold across the group's warps (xch: 2*NW values of shared scratch), then fixed up.
template <typename T, int M, int NW, class Sync = BlockSync<NW>>
__device__ __forceinline__ void group_apply_r(T (&v)[M], const T (&fi)[M], const T (&fa)[M], const T (&fb)[M], int t,
                                              T *xch, Sync sync = Sync())
{
    const int lane = t & (WARP - 1), wl = t / WARP;
    T gk[M];
    T y = T(0), g = T(1);
#pragma unroll
    for (int k = 0; k < M; k++) {
        T a = fa[k];
        y = fma_rn(a, y, mul_rn(fi[k], v[k]));
        v[k] = y;
        g = g * a;
        gk[k] = g;
    }
    T G = g, Y = y;
#pragma unroll
    for (int s = 1; s < WARP; s <<= 1) {
        T Gp = shfl_up(G, s), Yp = shfl_up(Y, s);
        if (lane >= s) { Y = Y + G * Yp; G = G * Gp; }
    }
    T yw = T(0);
    if (NW > 1) {
        if (lane == WARP - 1) { xch[2 * wl] = G; xch[2 * wl + 1] = Y; }
        sync();
        for (int w2 = 0; w2 < wl; w2++) yw = xch[2 * w2 + 1] + xch[2 * w2] * yw;
        sync();
    }
    {
        T Yp = shfl_up(Y, 1), Gp = shfl_up(G, 1);
        T yin = (lane == 0) ? yw : Yp + Gp * yw;
#pragma unroll
        for (int k = 0; k < M; k++) v[k] = v[k] + gk[k] * yin;
    }
    T x = T(0), h = T(1);
#pragma unroll
    for (int k = M - 1; k >= 0; k--) {
        T b = fb[k];
        x = v[k] + b * x;
        v[k] = x;
        h = h * b;
        gk[k] = h;
    }
    T H = h, X = x;
#pragma unroll
    for (int s = 1; s < WARP; s <<= 1) {
        T Hn = shfl_down(H, s), Xn = shfl_down(X, s);
        if (lane + s < WARP) { X = X + H * Xn; H = H * Hn; }
    }
    T xw = T(0);
    if (NW > 1) {
        if (lane == 0) { xch[2 * wl] = H; xch[2 * wl + 1] = X; }
        sync();
        for (int w2 = NW - 1; w2 > wl; w2--) xw = xch[2 * w2 + 1] + xch[2 * w2] * xw;
        sync();
    }
    {
        T Xn = shfl_down(X, 1), Hn = shfl_down(H, 1);
        T xin = (lane == WARP - 1) ? xw : Xn + Hn * xw;
#pragma unroll
        for (int k = 0; k < M; k++) v[k] = v[k] + gk[k] * xin;
    }
}

// Load the factors of one line (chunk ownership) into registers.
template <typename T, int M, int NW>
__device__ __forceinline__ void load_factors(T (&fi)[M], T (&fa)[M], T (&fb)[M], const T *__restrict__ invD,
                                             const T *__restrict__ pa, const T *__restrict__ pb, int t)
{
    constexpr int TG = WARP * NW;
#pragma unroll
    for (int k = 0; k < M; k++) {
        fi[k] = invD[k * TG + t];
        fa[k] = pa[k * TG + t];
        fb[k] = pb[k * TG + t];
    }
}

template <typename T, int M, int NW>
__device__ __forceinline__ void group_apply(T (&v)[M], const T *__restrict__ invD, const T *__restrict__ fa,
                                            const T *__restrict__ fb, int t, T *xch)
{
    T ri[M], ra[M], rb[M];
    load_factors<T, M, NW>(ri, ra, rb, invD, fa, fb, t);
    group_apply_r<T, M, NW>(v, ri, ra, rb, t, xch);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while its predecessor finishes; it must not read the
// predecessor's results (or write anything the predecessor reads) before
// griddep_wait().  griddep_launch() lets the successor start its own prologue.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Sherman-Morrison completion of a cyclic line after group_apply on the modified
// matrix (chunk ownership): x = y - ((y_1 + cv*y_n) * sinv) z.  xch: 2 values.
template <typename T, int M, int NW>
__device__ __forceinline__ void group_cyclic_fix(T (&v)[M], const T *__restrict__ z, T cv, T sinv, int n, int t,
                                                 T *xch)
{
    constexpr int TG = WARP * NW;
    const int last = n - 1, tl = last / M, kl = last % M;
    if (t == 0) xch[0] = v[0];
    if (t == tl) {
#pragma unroll
        for (int k = 0; k < M; k++)
            if (k == kl) xch[1] = v[k];
    }
    gsync<NW>();
    T w = (xch[0] + cv * xch[1]) * sinv;
    gsync<NW>();
#pragma unroll
    for (int k = 0; k < M; k++) v[k] = v[k] - w * z[k * TG + t];
}

// Group geometry of a line kernel launched with 128-thread blocks: 4/NW lines per
// block; returns the group's line index and the thread index inside the group.
template <int NW>
__device__ __forceinline__ void group_of(int &gline, int &t, int &gib)
{
    constexpr int TG = WARP * NW;
    gib = threadIdx.x / TG;
    t = threadIdx.x % TG;
    gline = blockIdx.x * (128 / TG) + gib;
}

// Host dispatch over the (elements per thread, warps per group) instantiations of a
// line kernel: f(std::integral_constant<int,M>, std::integral_constant<int,NW>).
template <typename F>
inline bool dispatch_line(const LineSys &s, F &&f)
{
    using std::integral_constant;
    switch (s.NW * 32 + s.M) {
#define FVM_LCASE(NWV, MV) \
    case NWV * 32 + MV: f(integral_constant<int, MV>(), integral_constant<int, NWV>()); return true;
        FVM_LCASE(1, 1) FVM_LCASE(1, 2) FVM_LCASE(1, 3) FVM_LCASE(1, 4)
        FVM_LCASE(1, 6) FVM_LCASE(1, 8) FVM_LCASE(1, 12)
        FVM_LCASE(2, 1) FVM_LCASE(2, 2) FVM_LCASE(2, 3) FVM_LCASE(2, 4) FVM_LCASE(2, 6) FVM_LCASE(2, 8)
        FVM_LCASE(4, 1) FVM_LCASE(4, 2) FVM_LCASE(4, 3) FVM_LCASE(4, 4)
#undef FVM_LCASE
    default: return false;
    }
}

// Launch with programmatic stream serialization (captured into graphs as
// programmatic edges): the kernel may begin while the preceding kernel drains.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// Line tiles with a kernel instantiation: NW warps per line (1, 2, 4) and M
// elements per thread (1..4; also 6, 8, 12 for one warp and 6, 8 for two).
inline bool tile_supported(int nw, int m)
{
    if (nw == 4) return m >= 1 && m <= 4;
    if (nw == 2) return (m >= 1 && m <= 4) || m == 6 || m == 8;
    if (nw == 1) return (m >= 1 && m <= 4) || m == 6 || m == 8 || m == 12;
    return false;
}

// Blocks of 128 threads needed for `lines` line groups of NW warps.
inline int line_blocks(int lines, int NW) { return (lines * NW + 3) / 4; }

// Threads per line group for a line of n unknowns (elements per thread <= 4 for
// n <= 512): one warp up to 128 unknowns, two up to 256, else four.
inline int group_warps(int n) { return n <= 128 ? 1 : (n <= 256 ? 2 : 4); }

}  // namespace fvm
