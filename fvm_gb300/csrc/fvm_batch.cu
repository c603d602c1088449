// fvm_batch.cu -- many independent cylinder cases with different grids, Reynolds
// numbers and time steps advanced together.
//
// Each case is an ordinary context (its own device slab, geometry, factors and
// state, set up through the single-context entry points).  A batch keeps a device
// table of the cases' device views; every sub-step of the time step is one launch
// over all cases (grid z = case, x/y extents = the largest case, surplus blocks of
// smaller cases return at once), so small cases fill the GPU together.  The whole
// step -- including the Poisson iteration as a device-side while loop that ends
// when the last case has converged or reached its sweep cap -- is one CUDA graph,
// launched once per step; CALCCOEF records of every case and step stay on the
// device until the call returns.  The cases share the line tiles (warps per line
// group, elements per thread) of the radial and circumferential line families;
// fvm_batch_autotune times the candidate tiles on the batch itself.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "fvm_internal.cuh"

using fvm::BatchCtl;
using fvm::Dev;
using fvm::Tgt;

struct fvm_batch {
    int ncases = 0;
    std::vector<fvm_ctx *> cases;
    fvm_ctx shell;                    // stream, error text and launch counters of the batched launches
    cudaStream_t st2 = nullptr;       // capture stream of the Poisson loop body
    Dev *d_devs = nullptr;            // device table of the cases' views
    BatchCtl *d_bctl = nullptr;
    double *d_time = nullptr;         // per-case simulated time
    fvm_coeffs *d_hist = nullptr;     // records [step * ncases + case]
    fvm_coeffs *h_hist = nullptr;     // pinned copy
    int hist_cap = 0;                 // steps of record capacity
    cudaGraphExec_t graph = nullptr;  // one time step of every case
    int outer_kernels = 0, body_kernels = 0, body_sweeps = 0;
    Tgt t;
};

namespace {

int berr(fvm_batch *b, const std::string &why, int code = FVM_ERR_ARG)
{
    b->shell.err = why;
    return code;
}

bool same_run_options(const fvm_params &a, const fvm_params &b)
{
    return a.precision == b.precision && a.thermal == b.thermal && a.iter_t_bug == b.iter_t_bug &&
           a.res_every == b.res_every && a.refine_sweeps == b.refine_sweeps && a.device == b.device &&
           a.poisson_groups == b.poisson_groups && a.tile_r_warps == b.tile_r_warps && a.tile_r_m == b.tile_r_m &&
           a.tile_t_warps == b.tile_t_warps && a.tile_t_m == b.tile_t_m;
}

// A tile (warps, elements per thread) that covers lines of n unknowns.
void auto_tile(int n, int &nw, int &m)
{
    nw = fvm::group_warps(n);
    m = (n + 32 * nw - 1) / (32 * nw);
}

// Launch extents and shared options of the batch (maxima over the cases).
void make_target(fvm_batch *b)
{
    Tgt &t = b->t;
    fvm_ctx *c0 = b->cases[0];
    t = fvm::tgt_of(c0);
    t.c = &b->shell;
    t.st = b->shell.stream;
    t.one = nullptr;
    t.tab.devs = b->d_devs;
    t.nz = b->ncases;
    for (fvm_ctx *c : b->cases) {
        t.NI = std::max(t.NI, c->NI);
        t.NJ = std::max(t.NJ, c->NJ);
        t.n = std::max(t.n, c->n);
        t.nblk_res = std::max(t.nblk_res, c->nblk_res);
        t.nblk_res64 = std::max(t.nblk_res64, c->nblk_res64);
        t.nblk_mres = std::max(t.nblk_mres, c->nblk_mres);
    }
}

int upload_table(fvm_batch *b)
{
    fvm_ctx *sh = &b->shell;
    std::vector<Dev> devs(b->ncases);
    std::vector<double> times(b->ncases);
    for (int k = 0; k < b->ncases; k++) {
        devs[k] = b->cases[k]->d;
        devs[k].case_id = k;
        devs[k].bctl = b->d_bctl;
        devs[k].bhist = b->d_hist;
        devs[k].btime = b->d_time + k;
        times[k] = b->cases[k]->rtime;
    }
    // bound on residual intervals per step: every case stops at its sweep cap
    // (cap/per intervals, one more for the mixed path's first residual), and the
    // loop body in flight completes (`groups` intervals); plus slack
    const int per = b->t.mixed ? b->t.refine_sweeps : b->t.res_every;
    const int pg = b->cases[0]->p.poisson_groups;
    const int groups = pg > 0 ? pg : (32 + per - 1) / per;
    int cap = 0;
    for (fvm_ctx *c : b->cases) cap = std::max(cap, c->d.nswpp);
    BatchCtl ctl{0, b->ncases, 0, 0, 0, 0};
    ctl.max_bodies = cap / per + groups + 3;
    FVM_CUDA(sh, cudaMemcpyAsync(b->d_devs, devs.data(), sizeof(Dev) * b->ncases, cudaMemcpyHostToDevice, sh->stream));
    FVM_CUDA(sh, cudaMemcpyAsync(b->d_time, times.data(), sizeof(double) * b->ncases, cudaMemcpyHostToDevice,
                                 sh->stream));
    FVM_CUDA(sh, cudaMemcpyAsync(b->d_bctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, sh->stream));
    FVM_CUDA(sh, cudaStreamSynchronize(sh->stream));
    return FVM_OK;
}

int ensure_history(fvm_batch *b, int steps)
{
    if (steps <= b->hist_cap) return FVM_OK;
    fvm_ctx *sh = &b->shell;
    if (b->d_hist) cudaFree(b->d_hist);
    if (b->h_hist) cudaFreeHost(b->h_hist);
    b->d_hist = nullptr;
    b->h_hist = nullptr;
    b->hist_cap = 0;
    const size_t bytes = sizeof(fvm_coeffs) * size_t(steps) * b->ncases;
    FVM_CUDA(sh, cudaMalloc(&b->d_hist, bytes));
    FVM_CUDA(sh, cudaMallocHost(&b->h_hist, bytes));
    b->hist_cap = steps;
    return FVM_OK;
}

// Every case's setup work (on its own stream) is complete.
int sync_cases(fvm_batch *b)
{
    for (fvm_ctx *c : b->cases) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return berr(b, std::string("case stream: ") + cudaGetErrorString(e), FVM_ERR_CUDA);
    }
    return FVM_OK;
}

void drop_graph(fvm_batch *b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

// Capture one time step of every case: the launches before the Poisson loop, a
// while-conditional node whose body holds `groups` residual intervals of the
// batched Poisson iteration, and the launches after it.
int build_graph(fvm_batch *b)
{
    if (b->graph) return FVM_OK;
    fvm_ctx *sh = &b->shell;
    Tgt t = b->t;
    const int per = t.mixed ? t.refine_sweeps : t.res_every;
    const int groups = b->cases[0]->p.poisson_groups > 0 ? b->cases[0]->p.poisson_groups : (32 + per - 1) / per;
    cudaStream_t st = sh->stream;
    cudaGraph_t g = nullptr;
    FVM_CUDA(sh, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    sh->capturing = true;
    sh->pgraph_kernels = 0;
    int rc = fvm::step_before_poisson(t);
    const int before = sh->pgraph_kernels;
    cudaError_t e = cudaSuccess;
    cudaGraphConditionalHandle h{};
    if (rc == FVM_OK) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        size_t nd = 0;
        e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &nd);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &cp);
        if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(b->st2, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            Tgt tb = t;
            tb.st = b->st2;
            rc = fvm::poisson_bodies(tb, h, 1, groups);
            cudaGraph_t body = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(b->st2, &body);
            if (e2 != cudaSuccess && rc == FVM_OK) e = e2;
        }
    }
    const int body = sh->pgraph_kernels - before;
    if (rc == FVM_OK && e == cudaSuccess) rc = fvm::step_after_poisson(t, 0.0, nullptr);
    if (rc == FVM_OK && e == cudaSuccess) rc = fvm::launch_batch_tick(t, b->d_bctl);
    sh->capturing = false;
    cudaError_t e3 = cudaStreamEndCapture(st, &g);
    if (rc != FVM_OK || e != cudaSuccess || e3 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (rc != FVM_OK) return rc;
        return berr(b, std::string("batch step capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e3),
                    FVM_ERR_CUDA);
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return berr(b, std::string("batch step instantiate: ") + cudaGetErrorString(e), FVM_ERR_CUDA);
    }
    b->body_kernels = body;
    b->outer_kernels = sh->pgraph_kernels - body;
    b->body_sweeps = groups * per;
    return FVM_OK;
}

// Give every case the tiles and recompute its factors; the step graph is rebuilt.
int apply_tiles(fvm_batch *b, int rw, int rm, int tw, int tm)
{
    for (fvm_ctx *c : b->cases) {
        if (32 * rw * rm < c->NI - 1 || 32 * tw * tm < c->NJ - 1)
            return berr(b, "line tile does not cover every case's lines");
    }
    for (fvm_ctx *c : b->cases) {
        c->p.tile_r_warps = rw;
        c->p.tile_r_m = rm;
        c->p.tile_t_warps = tw;
        c->p.tile_t_m = tm;
        if (c->pgraph) cudaGraphExecDestroy(c->pgraph);
        c->pgraph = nullptr;
        int rc = fvm::setup_factors(c);
        if (rc != FVM_OK) return berr(b, c->err, rc);
    }
    int rc = sync_cases(b);
    if (rc) return rc;
    drop_graph(b);
    make_target(b);
    return upload_table(b);
}

// Average time of one batched sweep pair (both colours) of `what` (0: Poisson,
// 1: circumferential predictor lines of U), replayed in a graph.
int time_kernels(fvm_batch *b, int what, int sweeps, double *ms)
{
    fvm_ctx *sh = &b->shell;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    FVM_CUDA(sh, cudaStreamBeginCapture(sh->stream, cudaStreamCaptureModeThreadLocal));
    sh->capturing = true;
    int rc = what == 0 ? fvm::sweep_pairs(b->t, sweeps) : fvm::theta_pairs(b->t, FVM_FIELD_U, sweeps);
    sh->capturing = false;
    cudaError_t e = cudaStreamEndCapture(sh->stream, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : berr(b, std::string("timing capture: ") + cudaGetErrorString(e), FVM_ERR_CUDA);
    }
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return berr(b, std::string("timing instantiate: ") + cudaGetErrorString(e), FVM_ERR_CUDA);
    FVM_CUDA(sh, cudaGraphLaunch(ge, sh->stream));   // warm
    FVM_CUDA(sh, cudaEventRecord(sh->ev_a, sh->stream));
    FVM_CUDA(sh, cudaGraphLaunch(ge, sh->stream));
    FVM_CUDA(sh, cudaEventRecord(sh->ev_b, sh->stream));
    FVM_CUDA(sh, cudaEventSynchronize(sh->ev_b));
    float t_ms = 0.f;
    FVM_CUDA(sh, cudaEventElapsedTime(&t_ms, sh->ev_a, sh->ev_b));
    cudaGraphExecDestroy(ge);
    *ms = t_ms / sweeps;
    return FVM_OK;
}

}  // namespace

extern "C" {

int fvm_batch_create(int ncases, const fvm_params *params, fvm_batch **out)
{
    if (!out) return FVM_ERR_ARG;
    *out = nullptr;
    if (ncases < 1 || !params) return FVM_ERR_ARG;
    for (int k = 1; k < ncases; k++)
        if (!same_run_options(params[0], params[k])) return FVM_ERR_ARG;
    fvm_batch *b = new (std::nothrow) fvm_batch();
    if (!b) return FVM_ERR_NOMEM;
    b->ncases = ncases;
    // shared tiles: given, or the automatic tile of the longest line of each family
    int rw = params[0].tile_r_warps, rm = params[0].tile_r_m, tw = params[0].tile_t_warps, tm = params[0].tile_t_m;
    if (rw == 0 && rm == 0) {
        int nmax = 0;
        for (int k = 0; k < ncases; k++) nmax = std::max(nmax, params[k].ni - 1);
        auto_tile(nmax, rw, rm);
    }
    if (tw == 0 && tm == 0) {
        int nmax = 0;
        for (int k = 0; k < ncases; k++) nmax = std::max(nmax, params[k].nj - 1);
        auto_tile(nmax, tw, tm);
    }
    fvm_ctx *sh = &b->shell;
    sh->p = params[0];
    cudaError_t e = cudaSetDevice(params[0].device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sh->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->st2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&sh->ev_a);
    if (e == cudaSuccess) e = cudaEventCreate(&sh->ev_b);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_devs, sizeof(Dev) * ncases);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_bctl, sizeof(BatchCtl));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_time, sizeof(double) * ncases);
    if (e != cudaSuccess) {
        fvm_batch_destroy(b);
        return FVM_ERR_CUDA;
    }
    for (int k = 0; k < ncases; k++) {
        fvm_params p = params[k];
        p.tile_r_warps = rw;
        p.tile_r_m = rm;
        p.tile_t_warps = tw;
        p.tile_t_m = tm;
        fvm_ctx *c = nullptr;
        int rc = fvm_create(&p, &c);
        if (rc != FVM_OK) {
            fvm_batch_destroy(b);
            return rc;
        }
        b->cases.push_back(c);
    }
    make_target(b);
    *out = b;
    return FVM_OK;
}

int fvm_batch_destroy(fvm_batch *b)
{
    if (!b) return FVM_ERR_ARG;
    if (b->shell.stream) cudaStreamSynchronize(b->shell.stream);
    drop_graph(b);
    for (fvm_ctx *c : b->cases) fvm_destroy(c);
    if (b->d_devs) cudaFree(b->d_devs);
    if (b->d_bctl) cudaFree(b->d_bctl);
    if (b->d_time) cudaFree(b->d_time);
    if (b->d_hist) cudaFree(b->d_hist);
    if (b->h_hist) cudaFreeHost(b->h_hist);
    if (b->shell.ev_a) cudaEventDestroy(b->shell.ev_a);
    if (b->shell.ev_b) cudaEventDestroy(b->shell.ev_b);
    if (b->st2) cudaStreamDestroy(b->st2);
    if (b->shell.stream) cudaStreamDestroy(b->shell.stream);
    delete b;
    return FVM_OK;
}

const char *fvm_batch_last_error(const fvm_batch *b)
{
    if (!b) return "null batch";
    return b->shell.err.c_str();
}

int fvm_batch_case(fvm_batch *b, int k, fvm_ctx **ctx)
{
    if (!b || !ctx || k < 0 || k >= b->ncases) return FVM_ERR_ARG;
    *ctx = b->cases[k];
    return FVM_OK;
}

int fvm_batch_tiles(const fvm_batch *b, int *tiles)
{
    if (!b || !tiles) return FVM_ERR_ARG;
    const fvm_params &p = b->cases[0]->p;
    tiles[0] = p.tile_r_warps;
    tiles[1] = p.tile_r_m;
    tiles[2] = p.tile_t_warps;
    tiles[3] = p.tile_t_m;
    return FVM_OK;
}

int fvm_batch_set_tiles(fvm_batch *b, const int *tiles)
{
    if (!b || !tiles) return FVM_ERR_ARG;
    auto ok = [](int nw, int m) { return fvm::tile_supported(nw, m); };
    if (!ok(tiles[0], tiles[1]) || !ok(tiles[2], tiles[3])) return berr(b, "invalid line tile");
    return apply_tiles(b, tiles[0], tiles[1], tiles[2], tiles[3]);
}

int fvm_batch_autotune(fvm_batch *b, int sweeps, int *tiles, double *ms)
{
    if (!b || sweeps < 1) return FVM_ERR_ARG;
    for (fvm_ctx *c : b->cases)
        if (!c->grid_set) return berr(b, "autotune needs every case's grid");
    int nr = 0, nt = 0;
    for (fvm_ctx *c : b->cases) {
        nr = std::max(nr, c->NI - 1);
        nt = std::max(nt, c->NJ - 1);
    }
    // the flow state is kept: the timed kernels write only scratch (Poisson) or
    // the U field, which is saved and restored around the circumferential timing
    std::vector<double *> saved(b->ncases, nullptr);
    fvm_ctx *sh = &b->shell;
    int rc = sync_cases(b);
    if (rc) return rc;
    for (int k = 0; k < b->ncases; k++) {
        fvm_ctx *c = b->cases[k];
        FVM_CUDA(sh, cudaMalloc(&saved[k], sizeof(double) * c->n));
        FVM_CUDA(sh, cudaMemcpy(saved[k], c->d.U, sizeof(double) * c->n, cudaMemcpyDeviceToDevice));
    }
    int cur[4];
    fvm_batch_tiles(b, cur);
    int best[4] = {cur[0], cur[1], cur[2], cur[3]};
    double best_ms[2] = {1e30, 1e30};
    for (int fam = 0; fam < 2 && rc == FVM_OK; fam++) {
        const int n = fam == 0 ? nr : nt;
        for (int nw = 1; nw <= 4 && rc == FVM_OK; nw *= 2) {
            int m = (n + 32 * nw - 1) / (32 * nw);
            while (m <= 12 && !fvm::tile_supported(nw, m)) m++;   // the smallest instantiated tile that covers n
            if (!fvm::tile_supported(nw, m)) continue;
            int tl[4] = {best[0], best[1], best[2], best[3]};
            tl[2 * fam] = nw;
            tl[2 * fam + 1] = m;
            rc = apply_tiles(b, tl[0], tl[1], tl[2], tl[3]);
            double t_ms = 0.0;
            if (rc == FVM_OK) rc = time_kernels(b, fam, sweeps, &t_ms);
            if (rc == FVM_OK && t_ms < best_ms[fam]) {
                best_ms[fam] = t_ms;
                best[2 * fam] = nw;
                best[2 * fam + 1] = m;
            }
        }
    }
    if (rc == FVM_OK) rc = apply_tiles(b, best[0], best[1], best[2], best[3]);
    for (int k = 0; k < b->ncases; k++) {
        if (!saved[k]) continue;
        if (rc == FVM_OK) {
            cudaError_t e = cudaMemcpy(b->cases[k]->d.U, saved[k], sizeof(double) * b->cases[k]->n,
                                       cudaMemcpyDeviceToDevice);
            if (e != cudaSuccess) rc = berr(b, cudaGetErrorString(e), FVM_ERR_CUDA);
        }
        cudaFree(saved[k]);
    }
    if (rc != FVM_OK) return rc;
    if (tiles) fvm_batch_tiles(b, tiles);
    if (ms) {
        ms[0] = best_ms[0];
        ms[1] = best_ms[1];
    }
    return FVM_OK;
}

int fvm_batch_time_sweeps(fvm_batch *b, int sweeps, double *ms_per_sweep)
{
    if (!b || sweeps < 1 || !ms_per_sweep) return FVM_ERR_ARG;
    int rc = sync_cases(b);
    if (rc == FVM_OK) rc = upload_table(b);
    if (rc == FVM_OK) rc = time_kernels(b, 0, sweeps, ms_per_sweep);
    return rc;
}

int fvm_batch_step(fvm_batch *b, int nsteps, fvm_coeffs *out)
{
    if (!b || nsteps < 1) return FVM_ERR_ARG;
    for (fvm_ctx *c : b->cases)
        if (!c->init_done) return berr(b, "every case needs fvm_init (or fvm_upload_state) before stepping");
    fvm_ctx *sh = &b->shell;
    int rc = sync_cases(b);
    if (rc == FVM_OK) rc = ensure_history(b, nsteps);
    if (rc == FVM_OK) rc = upload_table(b);
    if (rc == FVM_OK) rc = build_graph(b);
    if (rc) return rc;
    for (int s = 0; s < nsteps; s++) FVM_CUDA(sh, cudaGraphLaunch(b->graph, sh->stream));
    const size_t cnt = size_t(nsteps) * b->ncases;
    FVM_CUDA(sh, cudaMemcpyAsync(b->h_hist, b->d_hist, sizeof(fvm_coeffs) * cnt, cudaMemcpyDeviceToHost, sh->stream));
    BatchCtl ctl{};
    FVM_CUDA(sh, cudaMemcpyAsync(&ctl, b->d_bctl, sizeof(ctl), cudaMemcpyDeviceToHost, sh->stream));
    FVM_CUDA(sh, cudaStreamSynchronize(sh->stream));
    if (ctl.overrun) return berr(b, "batched Poisson loop ended by its iteration bound", FVM_ERR_TIMEOUT);
    int status = FVM_OK;
    const bool mixed = b->t.mixed;
    long long bodies = 0;   // loop bodies launched: set by the slowest case of each step
    for (int s = 0; s < nsteps; s++) {
        int mx = 0;
        for (int k = 0; k < b->ncases; k++) mx = std::max(mx, b->h_hist[size_t(s) * b->ncases + k].sweeps);
        bodies += std::max(1, (mx + (mixed ? 1 : 0) + b->body_sweeps - 1) / b->body_sweeps);
    }
    for (int k = 0; k < b->ncases; k++) {
        fvm_ctx *c = b->cases[k];
        c->hist.clear();
        for (int s = 0; s < nsteps; s++) {
            const fvm_coeffs &co = b->h_hist[size_t(s) * b->ncases + k];
            c->hist.push_back(co);
            c->tm.sweeps += co.sweeps;
            c->tm.steps++;
            if (!std::isfinite(co.resid) || !std::isfinite(co.cd) || !std::isfinite(co.cl)) {
                b->shell.err = "non-finite Poisson residual, drag or lift in case " + std::to_string(k);
                status = FVM_ERR_NAN;
            } else if (co.resid > c->p.resimax && status == FVM_OK) {
                status = FVM_ERR_NOCONV;
            }
        }
        c->last = c->hist.back();
        c->rtime = c->last.time;
        c->niter_time += nsteps;
    }
    if (out) std::memcpy(out, b->h_hist, sizeof(fvm_coeffs) * cnt);
    sh->tm.kernel_launches += (long long)nsteps * b->outer_kernels + bodies * b->body_kernels;
    sh->tm.steps += nsteps;
    return status;
}

int fvm_batch_get_timing(const fvm_batch *b, fvm_timing *out)
{
    if (!b || !out) return FVM_ERR_ARG;
    *out = b->shell.tm;
    return FVM_OK;
}

}  // extern "C"
