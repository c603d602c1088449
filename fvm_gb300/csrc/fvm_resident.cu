// fvm_resident.cu -- line-resident zebra sweeps of the FP32 Poisson correction
// (mixed precision): one launch runs a whole refinement interval.
//
// The per-colour path launches one grid per zebra colour (two per sweep), and each
// launch re-reads its line factors, couplings and right-hand side from L2.  Here
// the radial lines j = 1..NJ-1 are split into blocks of B consecutive lines (B
// even); each CTA keeps its lines' FP32 factors, couplings, right-hand side and
// current correction on chip (registers and shared memory) for all refine_sweeps
// sweeps of the interval, so a sweep moves nothing but the boundary lines between
// neighbouring CTAs.
//
// Zebra order (odd lines, then even lines; lisolv.f90:18-33 reordered as in the
// per-colour kernels, neighbours through the periodic branch cut).  A CTA owning
// lines j0 .. j0+B-1 (j0 odd) also solves line j0+B, the first (odd) line of the
// next CTA, redundantly in the odd half: its even line j0+B-1 then finds both
// neighbours on chip, and the only data from other CTAs a sweep needs are the
// previous sweep's values of line j0-1 (last line of the CTA before) and of line
// j0+B+1 (second line of the CTA after).  One exchange per sweep, both directions
// at once.  The redundant line's result is bit-identical to its owner's (same
// inputs, same code).
//
// Exchange without flags or fences: every published element is one 64-bit word
// (FP32 value bits | tag << 32) written and polled with relaxed gpu-scope 64-bit
// accesses (single-copy atomic), so a word whose tag matches carries the value of
// that sweep.  Tags are the CTA's count of completed sweeps (kept in XCNT across
// launches, equal in every CTA), words alternate between two slots by sweep
// parity, and a slot is overwritten only after both readers have passed the sweep
// that read it.  Every wait is bounded (max_polls); a wait that runs out sets the
// control block's fault flag, ends the Poisson loop and returns, and the host
// reports FVM_ERR_TIMEOUT and clears the exchange state.
//
// The arithmetic of a line (right-hand side, precomputed-factor solve, correction
// added to P in FP64 with the BCP ghosts refreshed) is the per-colour kernel's,
// operation for operation, so both paths give identical bits.  Compiled with
// -ftz=true, as the per-colour sweeps are.
//
// k_pois32_resident2 (below) exchanges once per two sweeps: 4-line blocks keep an
// 11-line window and solve the neighbours' three nearest lines again; and either
// kernel, launched inside the forward Poisson loop, first takes the loop's
// convergence decision from the residual kernel's block sums (resident_decide).
#include <type_traits>

#include "fvm_internal.cuh"
#include "fvm_ops.cuh"

namespace fvm {
namespace {

// volatile: re-executed on every poll; no memory clobber, so the loads of one poll
// can all be in flight at once
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ void st_word(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Convergence decision of the forward Poisson loop at the start of a resident
// launch (sys.decide): every block sums the block partials the residual kernel
// k_mres left, in that kernel's own order (the same bits in every block), and takes
// k_mres's decision (iter_p.f90:37-50: done once the scaled residual is at the
// tolerance or the sweeps reach the cap) with the loop's sweep count from its own
// XCNT; block 0 records it.  Returns true when the loop is done: the launch then
// does nothing.  This takes the last-block reduction off the residual kernel's
// critical path.
template <int HAS_COND>
__device__ bool resident_decide(const Dev &d, const ResSys &sys, int S, double *sh, cudaGraphConditionalHandle cond)
{
    double a, b;
    sum_partials256(d.partial, d.nblk_mres, a, b, sh);
    if (threadIdx.x == 0) sh[0] = a / b;   // warp 0 has finished reading sh
    __syncthreads();
    const double resip = sh[0];
    const int it = (int)(d.XCNT[blockIdx.x] - sys.pctl->xbase);
    const bool stop = it > 0 && !(resip > d.resimax && it < d.nswpp);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sys.pctl->resip = resip;
        if (stop) {
            sys.pctl->done = 1;
            sys.pctl->capped = (resip > d.resimax) ? 1 : 0;
            sys.pctl->niter = it;
            if (HAS_COND) cudaGraphSetConditional(cond, 0);
        } else {
            sys.pctl->niter = it + S;
        }
    }
    return stop;
}

// Shared memory of a block: the block's current line values (B+1 lines, LW words
// each) and one fold buffer per line group.  Every value of the block stays in the
// chunk ownership of the line solve (thread t of a group holds elements
// t*M .. t*M+M-1); a line is stored as word k*TG + t = element t*M + k, so a
// neighbouring group reads exactly the elements its own thread t needs, bank-
// conflict free, and no transpose is needed.
template <int M, int NW>
struct ResLayout {
    // block size bound: wide chunks (M >= 6) keep their values in up to 128
    // registers per thread, so their blocks stay within 512 threads
    static constexpr int MAXT = M >= 6 ? 512 : 1024;
    static constexpr int TG = WARP * NW;
    static constexpr int LW = TG * M;   // words per line
    static size_t bytes(int B) { return sizeof(float) * size_t(B + 1) * (LW + 2 * NW); }
    // largest block of this instantiation (the dynamic shared memory allowed for it)
    static size_t max_bytes() { return bytes(MAXT / TG - 1); }
};

// Lines j0 .. j0+B-1 of block blockIdx.x and the redundant line j0+B: group g
// (32*NW threads) owns line j0+g.  S sweeps; apply != 0 adds the correction to P
// afterwards.  check_done != 0 returns at once when the loop is already done.
template <int M, int NW, int HAS_COND>
__global__ void __launch_bounds__(ResLayout<M, NW>::MAXT, 1)
    k_pois32_resident(const __grid_constant__ Dev d, const __grid_constant__ ResSys sys, int B, int S, int apply,
                      int check_done, int max_polls, unsigned tag_skew, cudaGraphConditionalHandle cond)
{
    using Lay = ResLayout<M, NW>;
    constexpr int TG = Lay::TG, LW = Lay::LW;
    extern __shared__ float shm[];
    __shared__ int s_fault, s_stop;
    __shared__ double s_sum[64];
    float *lines = shm;
    const int g = threadIdx.x / TG, t = threadIdx.x % TG;
    float *xch = shm + size_t(B + 1) * LW + size_t(g) * 2 * NW;
    const NamedSync<NW> bar{1 + g};
    const int L = d.NJ - 1;
    const int j0 = blockIdx.x * B + 1;
    auto wrap = [L](int j) { return j < 1 ? j + L : (j > L ? j - L : j); };
    const int j = wrap(j0 + g);
    const int n = d.sP.n;
    if (threadIdx.x == 0) {   // the loop's done flag, read once for the whole block
        s_fault = 0;
        s_stop = check_done ? sys.pctl->done : 0;
    }
    __syncthreads();
    if (s_stop) return;
    if (sys.decide && resident_decide<HAS_COND>(d, sys, S, s_sum, cond)) return;

    const size_t base = size_t(j - 1) * LW;
    float fi[M], fa[M], fb[M], an[M], as[M], rf[M], v[M], halo[M];
    load_factors<float, M, NW>(fi, fa, fb, sys.invDf + base, sys.faf + base, sys.fbf + base, t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        const int e = t * M + k;   // chunk ownership
        const bool ok = e < n;
        const int c = IDX(e + 1, j);
        an[k] = ok ? sys.ANf[c] : 0.0f;
        as[k] = ok ? sys.ASf[c] : 0.0f;
        rf[k] = ok ? sys.RF[c] : 0.0f;
        halo[k] = 0.0f;   // the correction starts from zero
        v[k] = 0.0f;
        lines[g * LW + k * TG + t] = 0.0f;
    }
    const unsigned cnt0 = d.XCNT[blockIdx.x];
    const bool odd_line = (g & 1) == 0;            // j0 is odd: even g = colour 0
    const bool publish = g == 1 || g == B - 1;     // read by the blocks before / after
    const int hline = g == 0 ? wrap(j0 - 1) : (g == B ? wrap(j0 + B + 1) : 0);
    __syncthreads();

    int sw = 1;
    for (; sw <= S; sw++) {
        // odd lines (and the redundant first line of the next block)
        if (odd_line) {
            if (sw > 1 && hline) {
                const unsigned want = cnt0 + unsigned(sw - 1) + tag_skew;
                const unsigned long long *src = d.XW + (size_t((sw - 1) & 1) * L + (hline - 1)) * LW;
                unsigned pending = 0;
#pragma unroll
                for (int k = 0; k < M; k++)
                    if (t * M + k < n) pending |= 1u << k;
                for (int it = 0; pending && it < max_polls; it++) {
                    // one L2 round trip per poll: every pending word's load is issued
                    // before any is tested
                    unsigned long long w[M];
#pragma unroll
                    for (int k = 0; k < M; k++) w[k] = ((pending >> k) & 1u) ? ld_word(src + k * TG + t) : 0ull;
#pragma unroll
                    for (int k = 0; k < M; k++) {
                        if (((pending >> k) & 1u) && unsigned(w[k] >> 32) == want) {
                            halo[k] = __uint_as_float(unsigned(w[k]));
                            pending &= ~(1u << k);
                        }
                    }
                }
                if (pending) s_fault = 1;
            }
#pragma unroll
            for (int k = 0; k < M; k++) {
                const float xs = g == 0 ? halo[k] : lines[(g - 1) * LW + k * TG + t];
                const float xn = g == B ? halo[k] : lines[(g + 1) * LW + k * TG + t];
                v[k] = t * M + k < n ? pois32_rhs(an[k], xn, as[k], xs, rf[k]) : 0.0f;
            }
            group_apply_r<float, M, NW>(v, fi, fa, fb, t, xch, bar);
#pragma unroll
            for (int k = 0; k < M; k++) lines[g * LW + k * TG + t] = v[k];
        }
        __syncthreads();
        if (s_fault) break;   // read by every thread after the barrier: a uniform exit
        // even lines: both neighbours are on chip
        if (!odd_line) {
#pragma unroll
            for (int k = 0; k < M; k++) {
                const float xs = lines[(g - 1) * LW + k * TG + t];
                const float xn = lines[(g + 1) * LW + k * TG + t];
                v[k] = t * M + k < n ? pois32_rhs(an[k], xn, as[k], xs, rf[k]) : 0.0f;
            }
            group_apply_r<float, M, NW>(v, fi, fa, fb, t, xch, bar);
#pragma unroll
            for (int k = 0; k < M; k++) lines[g * LW + k * TG + t] = v[k];
            if (publish) {
                unsigned long long *dst = d.XW + (size_t(sw & 1) * L + (j - 1)) * LW;
                const unsigned long long tag = (unsigned long long)(cnt0 + unsigned(sw)) << 32;
#pragma unroll
                for (int k = 0; k < M; k++)
                    if (t * M + k < n) st_word(dst + k * TG + t, tag | __float_as_uint(v[k]));
            }
        }
        __syncthreads();
    }

    // the next residual launch (programmatic) may start its coefficient prologue;
    // it reads P only after its dependency wait, i.e. after this grid has finished
    griddep_launch();
    if (sw <= S) {   // a wait ran out: end the loop, leave P alone
        if (threadIdx.x == 0) {
            sys.pctl->fault = 1;
            sys.pctl->done = 1;
            if (HAS_COND) cudaGraphSetConditional(cond, 0);
        }
        return;
    }
    if (g < B) {
#pragma unroll
        for (int k = 0; k < M; k++) {
            const int e = t * M + k;
            if (e < n) sys.DF[IDX(e + 1, j)] = v[k];
        }
        if (apply) {
#pragma unroll
            for (int k = 0; k < M; k++) {
                const int e = t * M + k;
                if (e < n) sys.X[IDX(e + 1, j)] += (double)v[k];
            }
            if (sys.bcp) {
                bar();
                if (t < WARP) refresh_row_ghosts<BCK_POISSON>(d, sys.X, sys.X, j, nullptr, nullptr, t);
            }
        }
    }
    if (threadIdx.x == 0) d.XCNT[blockIdx.x] = cnt0 + unsigned(S);
}

// Two sweeps per exchange.  A block of B = 4 lines j0 .. j0+3 keeps the window of
// lines j0-3 .. j0+B+3 on chip (rows w = 0 .. B+6, line j0-3+w; odd lines are the
// odd rows) and solves rows 1 .. B+5, one line group each.  A pair of sweeps starts
// from the previous sweep's values of the window's even lines; in the pair's first
// sweep the odd rows 1 .. B+5 and then the even rows 2 .. B+4 are solved, in the
// second the odd rows 3 .. B+3 and the even rows 4 .. B+2 (the block's own even
// lines): each half-sweep needs both neighbours, so the valid part of the window
// narrows by one row per half.  The rows beyond the block's own are the
// neighbours' lines solved again here with the same inputs and code, so their bits
// equal the owners'.  The only data from other blocks are the window's outer even
// rows 0, 2 and B+4, B+6, which are the even lines of the blocks before and after:
// every block publishes its two even lines once per pair and polls four lines at
// the start of the next, so one exchange serves two sweeps.  Tags and slots as in
// k_pois32_resident, counted per pair.
template <int M, int NW>
struct ResLayout2 {
    static constexpr int B = 4;
    static constexpr int TG = WARP * NW;
    static constexpr int LW = TG * M;
    static constexpr int NL = B + 7;   // window rows
    static constexpr int NG = B + 5;   // line groups (rows 1 .. B+5)
    static constexpr int NT = NG * TG;
    static size_t bytes() { return sizeof(float) * (size_t(NL) * LW + size_t(NG) * 2 * NW); }
};

template <int M, int NW, int HAS_COND>
__global__ void __launch_bounds__(ResLayout2<M, NW>::NT, 1)
    k_pois32_resident2(const __grid_constant__ Dev d, const __grid_constant__ ResSys sys, int S, int apply,
                       int check_done, int max_polls, unsigned tag_skew, cudaGraphConditionalHandle cond)
{
    using Lay = ResLayout2<M, NW>;
    constexpr int TG = Lay::TG, LW = Lay::LW, B = Lay::B, NL = Lay::NL;
    extern __shared__ float shm[];
    __shared__ int s_fault, s_stop;
    __shared__ double s_sum[64];
    float *rows = shm;
    const int gi = threadIdx.x / TG, t = threadIdx.x % TG;
    const int w = gi + 1;   // the window row this group solves
    float *xch = shm + size_t(NL) * LW + size_t(gi) * 2 * NW;
    const NamedSync<NW> bar{1 + gi};
    const int L = d.NJ - 1;
    const int j0 = blockIdx.x * B + 1;
    auto wrap = [L](int j) { return j < 1 ? j + L : (j > L ? j - L : j); };
    const int j = wrap(j0 - 3 + w);
    const int n = d.sP.n;
    if (threadIdx.x == 0) {
        s_fault = 0;
        s_stop = check_done ? sys.pctl->done : 0;
    }
    __syncthreads();
    if (s_stop) return;
    if (sys.decide && resident_decide<HAS_COND>(d, sys, S, s_sum, cond)) return;

    const size_t base = size_t(j - 1) * LW;
    float fi[M], fa[M], fb[M], an[M], as[M], rf[M], v[M];
    load_factors<float, M, NW>(fi, fa, fb, sys.invDf + base, sys.faf + base, sys.fbf + base, t);
#pragma unroll
    for (int k = 0; k < M; k++) {
        const int e = t * M + k;
        const bool ok = e < n;
        const int c = IDX(e + 1, j);
        an[k] = ok ? sys.ANf[c] : 0.0f;
        as[k] = ok ? sys.ASf[c] : 0.0f;
        rf[k] = ok ? sys.RF[c] : 0.0f;
        v[k] = 0.0f;
    }
    for (int q = threadIdx.x; q < NL * LW; q += Lay::NT) rows[q] = 0.0f;   // the correction starts from zero
    const unsigned cnt0 = d.XCNT[blockIdx.x];
    const bool odd = (w & 1) != 0;
    // the outer even rows, each polled by the group next to it
    const int hrow = w == 1 ? 0 : (w == 3 ? 2 : (w == B + 3 ? B + 4 : (w == B + 5 ? B + 6 : -1)));
    const int hline = hrow >= 0 ? wrap(j0 - 3 + hrow) : 0;
    const bool publish = !odd && w >= 4 && w <= B + 2;
    __syncthreads();

    auto solve = [&]() {
#pragma unroll
        for (int k = 0; k < M; k++) {
            const float xs = rows[(w - 1) * LW + k * TG + t];
            const float xn = rows[(w + 1) * LW + k * TG + t];
            v[k] = t * M + k < n ? pois32_rhs(an[k], xn, as[k], xs, rf[k]) : 0.0f;
        }
        group_apply_r<float, M, NW>(v, fi, fa, fb, t, xch, bar);
#pragma unroll
        for (int k = 0; k < M; k++) rows[w * LW + k * TG + t] = v[k];
    };

    int sw = 1;
    for (; sw <= S; sw += 2) {   // sweeps sw and sw+1
        if (sw > 1 && hrow >= 0) {
            const unsigned want = cnt0 + unsigned(sw - 1) + tag_skew;
            const unsigned long long *src = d.XW + (size_t(((sw - 1) >> 1) & 1) * L + (hline - 1)) * LW;
            unsigned pending = 0;
#pragma unroll
            for (int k = 0; k < M; k++)
                if (t * M + k < n) pending |= 1u << k;
            for (int it = 0; pending && it < max_polls; it++) {
                unsigned long long wd[M];
#pragma unroll
                for (int k = 0; k < M; k++) wd[k] = ((pending >> k) & 1u) ? ld_word(src + k * TG + t) : 0ull;
#pragma unroll
                for (int k = 0; k < M; k++) {
                    if (((pending >> k) & 1u) && unsigned(wd[k] >> 32) == want) {
                        rows[hrow * LW + k * TG + t] = __uint_as_float(unsigned(wd[k]));
                        pending &= ~(1u << k);
                    }
                }
            }
            if (pending) s_fault = 1;
        }
        __syncthreads();
        if (s_fault) break;   // uniform: read by every thread after the barrier
        if (odd) solve();                                  // sweep sw, odd rows 1 .. B+5
        __syncthreads();
        if (!odd) solve();                                 // sweep sw, even rows 2 .. B+4
        __syncthreads();
        if (odd && w >= 3 && w <= B + 3) solve();          // sweep sw+1, odd rows 3 .. B+3
        __syncthreads();
        if (publish) {                                     // sweep sw+1, the block's even lines
            solve();
            unsigned long long *dst = d.XW + (size_t(((sw + 1) >> 1) & 1) * L + (j - 1)) * LW;
            const unsigned long long tag = (unsigned long long)(cnt0 + unsigned(sw + 1)) << 32;
#pragma unroll
            for (int k = 0; k < M; k++)
                if (t * M + k < n) st_word(dst + k * TG + t, tag | __float_as_uint(v[k]));
        }
        __syncthreads();
    }

    // the next residual launch (programmatic) may start its coefficient prologue;
    // it reads P only after its dependency wait, i.e. after this grid has finished
    griddep_launch();
    if (sw <= S) {   // a wait ran out: end the loop, leave P alone
        if (threadIdx.x == 0) {
            sys.pctl->fault = 1;
            sys.pctl->done = 1;
            if (HAS_COND) cudaGraphSetConditional(cond, 0);
        }
        return;
    }
    if (w >= 3 && w <= B + 2) {   // the block's own lines
#pragma unroll
        for (int k = 0; k < M; k++) {
            const int e = t * M + k;
            if (e < n) sys.DF[IDX(e + 1, j)] = v[k];
        }
        if (apply) {
#pragma unroll
            for (int k = 0; k < M; k++) {
                const int e = t * M + k;
                if (e < n) sys.X[IDX(e + 1, j)] += (double)v[k];
            }
            if (sys.bcp) {
                bar();
                if (t < WARP) refresh_row_ghosts<BCK_POISSON>(d, sys.X, sys.X, j, nullptr, nullptr, t);
            }
        }
    }
    if (threadIdx.x == 0) d.XCNT[blockIdx.x] = cnt0 + unsigned(S);
}

template <int M, int NW, int HAS_COND>
cudaError_t launch_resident2(const fvm_ctx *c, const ResSys &sys, cudaStream_t st, int S, int apply, int check_done,
                             int max_polls, unsigned skew, cudaGraphConditionalHandle cond)
{
    using Lay = ResLayout2<M, NW>;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c->res_blocks);
    cfg.blockDim = dim3(Lay::NT);
    cfg.dynamicSmemBytes = Lay::bytes();
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = c->res_coop ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_pois32_resident2<M, NW, HAS_COND>, c->d, sys, S, apply, check_done, max_polls,
                              skew, cond);
}

template <int M, int NW, int HAS_COND>
cudaError_t launch_resident(const fvm_ctx *c, const ResSys &sys, cudaStream_t st, int S, int apply, int check_done,
                            int max_polls, unsigned skew, cudaGraphConditionalHandle cond)
{
    using Lay = ResLayout<M, NW>;
    auto k = k_pois32_resident<M, NW, HAS_COND>;
    const size_t smem = Lay::bytes(c->res_lines);   // allowed by resident_setup
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c->res_blocks);
    cfg.blockDim = dim3((c->res_lines + 1) * Lay::TG);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = c->res_coop ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, c->d, sys, c->res_lines, S, apply, check_done, max_polls, skew, cond);
}

}  // namespace

// Bounded wait of one exchange: about 1 s of polling at L2 latency.
constexpr int kResidentPolls = 1 << 21;

// Lines per block for the context (0: the per-colour path).  poisson_resident = 1
// takes 4 lines per block where they fit (measured fastest on 512 x 384: 2.40 us
// per sweep against 2.57 with 2), else the smallest even B dividing NJ-1 whose
// blocks are all co-resident; k >= 2 asks for k lines per block.
int resident_setup(fvm_ctx *c)
{
    c->res_lines = c->res_blocks = 0;
    c->res_coop = false;
    const int want = c->p.poisson_resident;
    if (c->p.precision != FVM_MIXED || want == 0) return FVM_OK;
    const LineSys &s = c->d.sP;
    const int L = c->NJ - 1, TG = WARP * s.NW;
    int sms = 0;
    FVM_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->p.device));
    const int order[] = {4, 2, 6, 8, 10, 12, 14};
    for (int B : order) {
        if (want >= 2 && B != want) continue;
        if (L % B || L / B < 2) continue;
        int per_sm = 0;
        cudaError_t e = cudaSuccess;
        bool ok = dispatch_line(s, [&](auto m, auto nw) {
            constexpr int M_ = decltype(m)::value, NW_ = decltype(nw)::value;
            if ((B + 1) * TG > ResLayout<M_, NW_>::MAXT) {
                e = cudaErrorInvalidConfiguration;
                return;
            }
            auto k0 = k_pois32_resident<M_, NW_, 0>;
            auto k1 = k_pois32_resident<M_, NW_, 1>;
            const size_t smem = ResLayout<M_, NW_>::bytes(B);
            // both variants may use the shared memory of their largest block (set here,
            // outside any stream capture; the same value for every context)
            const int cap = (int)ResLayout<M_, NW_>::max_bytes();
            e = cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
            if (e == cudaSuccess) e = cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k1, (B + 1) * TG, smem);
        });
        if (!ok || e != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (L / B <= per_sm * sms) {
            c->res_lines = B;
            c->res_blocks = L / B;
            c->res_coop = true;
            break;
        }
    }
    if (want >= 2 && !c->res_lines) {
        c->err = "poisson_resident: the requested lines per block do not divide NJ-1 into co-resident blocks";
        return FVM_ERR_ARG;
    }
    // two sweeps per exchange where the window fits: 4 lines per block, line groups
    // of one or two warps, at least three blocks around the ring, all co-resident
    c->res_depth = 1;
    if (c->res_lines == 4 && c->p.resident_depth != 1 && c->res_blocks >= 3) {
        cudaError_t e = cudaSuccess;
        dispatch_line(s, [&](auto m, auto nw) {
            constexpr int M_ = decltype(m)::value, NW_ = decltype(nw)::value;
            if constexpr (NW_ <= 2) {
                using Lay = ResLayout2<M_, NW_>;
                auto k0 = k_pois32_resident2<M_, NW_, 0>;
                auto k1 = k_pois32_resident2<M_, NW_, 1>;
                int per_sm = 0;
                e = cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Lay::bytes());
                if (e == cudaSuccess)
                    e = cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Lay::bytes());
                if (e == cudaSuccess)
                    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k1, Lay::NT, Lay::bytes());
                if (e == cudaSuccess && c->res_blocks <= per_sm * sms) c->res_depth = 2;
            }
        });
        if (e != cudaSuccess) cudaGetLastError();
    }
    if (c->p.resident_depth == 2 && c->res_depth != 2) {
        c->err = "resident_depth 2: needs 4 lines per block, line groups of at most two warps and 12 or more lines";
        return FVM_ERR_ARG;
    }
    return FVM_OK;
}

namespace {

// The forward pressure correction of a context.
ResSys forward_sys(const fvm_ctx *c)
{
    const Dev &d = c->d;
    return ResSys{d.sP.invDf, d.sP.faf, d.sP.fbf, d.cP.ANf, d.cP.ASf, d.RF, d.DF, d.P, d.pctl, 1, 0};
}

int launch_sys(fvm_ctx *c, const ResSys &sys, cudaStream_t st, int sweeps, int apply, int max_polls,
               unsigned tag_skew, cudaGraphConditionalHandle cond, int has_cond, int check_done)
{
    cudaError_t e = cudaErrorInvalidValue;
    const int polls = max_polls > 0 ? max_polls : kResidentPolls;
    const bool pairs = c->res_depth == 2 && sweeps % 2 == 0;   // two sweeps per exchange
    bool ok = dispatch_line(c->d.sP, [&](auto m, auto nw) {
        constexpr int M_ = decltype(m)::value, NW_ = decltype(nw)::value;
        if constexpr (NW_ <= 2) {
            if (pairs) {
                if (has_cond) e = launch_resident2<M_, NW_, 1>(c, sys, st, sweeps, apply, check_done, polls, tag_skew, cond);
                else e = launch_resident2<M_, NW_, 0>(c, sys, st, sweeps, apply, check_done, polls, tag_skew, cond);
                return;
            }
        }
        if (has_cond) e = launch_resident<M_, NW_, 1>(c, sys, st, sweeps, apply, check_done, polls, tag_skew, cond);
        else e = launch_resident<M_, NW_, 0>(c, sys, st, sweeps, apply, check_done, polls, tag_skew, cond);
    });
    if (!ok) {
        c->err = "line length above 512 cells is not supported";
        return FVM_ERR_ARG;
    }
    if (e != cudaSuccess) {
        c->err = std::string("resident sweep launch: ") + cudaGetErrorString(e);
        return FVM_ERR_CUDA;
    }
    KCOUNT(c);
    return FVM_OK;
}

}  // namespace

// One launch of the resident sweeps for a single context (batches use the
// per-colour path).  max_polls <= 0 takes the default bound.
int resident_sweeps(const Tgt &t, int sweeps, int apply, int max_polls, unsigned tag_skew,
                    cudaGraphConditionalHandle cond, int has_cond, int check_done, int decide)
{
    ResSys sys = forward_sys(t.c);
    sys.decide = decide;
    return launch_sys(t.c, sys, t.st, sweeps, apply, max_polls, tag_skew, cond, has_cond, check_done);
}

// The same sweeps on another system of the context's line tile (the adjoint's
// transposed Poisson equation); no graph condition, default wait bound.
int resident_sweeps_on(fvm_ctx *c, const ResSys &sys, int sweeps, int apply, int check_done)
{
    return launch_sys(c, sys, c->stream, sweeps, apply, 0, 0u, 0, 0, check_done);
}

// After a wait ran out: the blocks' sweep counts may disagree, so clear the
// exchange words, the counts and the fault flag (stream-ordered).
int resident_reset(fvm_ctx *c)
{
    const size_t words = 2 * size_t(c->NJ - 1) * WARP * 4 * 4;
    FVM_CUDA(c, cudaMemsetAsync(c->d.XW, 0, words * sizeof(unsigned long long), c->stream));
    FVM_CUDA(c, cudaMemsetAsync(c->d.XCNT, 0, size_t(c->NJ) * sizeof(unsigned int), c->stream));
    FVM_CUDA(c, cudaMemsetAsync(&c->d.pctl->fault, 0, sizeof(int), c->stream));
    return FVM_OK;
}

}  // namespace fvm
