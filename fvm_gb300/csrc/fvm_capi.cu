// fvm_capi.cu -- extern "C" entry points of include/fvm.h.  Every function checks
// its arguments and the call order, converts CUDA failures into status codes and
// never aborts.
#include <cmath>
#include <cstring>
#include <new>

#include "fvm_internal.cuh"

using fvm::Dev;

namespace {

int bad(fvm_ctx *c, const char *msg)
{
    if (c) c->err = msg;
    return FVM_ERR_ARG;
}

int need_ready(fvm_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) return bad(c, "fvm_set_grid has not been called");
    if (!c->init_done) return bad(c, "fvm_init (or fvm_upload_state) has not been called");
    return FVM_OK;
}

int check_params(const fvm_params *p, std::string &why)
{
    if (!p) { why = "null parameters"; return FVM_ERR_ARG; }
    if (p->ni < 5 || p->nj < 5) { why = "NI and NJ must be at least 5"; return FVM_ERR_ARG; }
    if ((p->nj - 1) % 2 != 0) { why = "NJ-1 (circumferential cells) must be even for the zebra order"; return FVM_ERR_ARG; }
    if (p->ni - 1 > 512 || p->nj - 1 > 512) { why = "at most 512 cells per line are supported"; return FVM_ERR_ARG; }
    if (!(p->dt > 0.0) || !(p->re > 0.0) || !(p->pr > 0.0)) { why = "dt, re and pr must be positive"; return FVM_ERR_ARG; }
    if (!(p->resimax >= 0.0) || p->nswpp < 1) { why = "resimax must be >= 0 and nswpp >= 1"; return FVM_ERR_ARG; }
    if (p->precision != FVM_FP64 && p->precision != FVM_MIXED) { why = "unknown precision"; return FVM_ERR_ARG; }
    auto tile_ok = [&](int nw, int m, int n, const char *fam) {
        if (nw == 0 && m == 0) return true;
        if (!fvm::tile_supported(nw, m) || 32 * nw * m < n) {
            why = std::string("invalid ") + fam + " line tile (warps 1, 2 or 4; 1..4 elements per thread, also "
                  "6, 8, 12 with one warp and 6, 8 with two; 32*warps*elements >= line length)";
            return false;
        }
        return true;
    };
    if (!tile_ok(p->tile_r_warps, p->tile_r_m, p->ni - 1, "radial")) return FVM_ERR_ARG;
    if (!tile_ok(p->tile_t_warps, p->tile_t_m, p->nj - 1, "circumferential")) return FVM_ERR_ARG;
    if (p->poisson_resident < 0 || (p->poisson_resident >= 2 && p->poisson_resident % 2)) {
        why = "poisson_resident: 0, 1 or an even number of lines per block";
        return FVM_ERR_ARG;
    }
    if (p->resident_depth < 0 || p->resident_depth > 2) {
        why = "resident_depth: 0 (automatic), 1 or 2 sweeps per exchange";
        return FVM_ERR_ARG;
    }
    return FVM_OK;
}

}  // namespace

extern "C" {

int fvm_default_params(fvm_params *p)
{
    if (!p) return FVM_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    p->ni = 97;
    p->nj = 129;
    p->re = 100.0;
    p->pr = 0.71;
    p->dt = 0.005;
    p->vel_rot = 0.0;
    p->uin = 1.0;      // comdat_param.f90:16-19
    p->vin = 0.0;
    p->tin = 0.0;
    p->t_wall = 1.0;
    p->resimax = 1.0e-4;  // comdat_param.f90:14
    p->nswpp = 20;        // comdat_param.f90:11
    p->precision = FVM_FP64;
    p->thermal = 1;
    p->iter_t_bug = 1;
    p->res_every = 1;
    p->refine_sweeps = 4;
    p->adi_refine = 2;
    p->device = 0;
    p->poisson_groups = 16;
    p->poisson_host_loop = 1;
    p->dd_positional = 1;
    p->poisson_resident = 1;
    return FVM_OK;
}

int fvm_create(const fvm_params *p, fvm_ctx **out)
{
    if (!out) return FVM_ERR_ARG;
    *out = nullptr;
    std::string why;
    if (check_params(p, why) != FVM_OK) return FVM_ERR_ARG;
    fvm_ctx *c = new (std::nothrow) fvm_ctx();
    if (!c) return FVM_ERR_NOMEM;
    c->p = *p;
    c->NI = p->ni;
    c->NJ = p->nj;
    c->NI1 = p->ni + 1;
    c->n = (p->ni + 1) * (p->nj + 1);
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_pctl, sizeof(fvm::PCtl));
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_a);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_b);
    if (e != cudaSuccess) {
        delete c;
        return FVM_ERR_CUDA;
    }
    int rc = fvm::setup_allocate(c);
    if (rc == FVM_OK) rc = fvm::resident_setup(c);
    if (rc != FVM_OK) {
        fvm_destroy(c);
        return rc;
    }
    *out = c;
    return FVM_OK;
}

int fvm_destroy(fvm_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    fvm::adj_destroy(c);
    fvm::post_free(c);
    if (c->pgraph) cudaGraphExecDestroy(c->pgraph);
    if (c->slab) cudaFree(c->slab);
    if (c->h_pctl) cudaFreeHost(c->h_pctl);
    if (c->ev_a) cudaEventDestroy(c->ev_a);
    if (c->ev_b) cudaEventDestroy(c->ev_b);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FVM_OK;
}

const char *fvm_last_error(const fvm_ctx *c)
{
    if (!c) return "null context";
    return c->err.c_str();
}

int fvm_set_grid(fvm_ctx *c, const double *xg, const double *yg)
{
    if (!c || !xg || !yg) return bad(c, "null grid pointer");
    const size_t bytes = sizeof(double) * c->n;
    FVM_CUDA(c, cudaMemcpyAsync(c->d.XG, xg, bytes, cudaMemcpyHostToDevice, c->stream));
    FVM_CUDA(c, cudaMemcpyAsync(c->d.YG, yg, bytes, cudaMemcpyHostToDevice, c->stream));
    int rc = fvm::setup_grid(c);
    if (rc == FVM_OK) c->grid_set = true;
    return rc;
}

int fvm_init(fvm_ctx *c, const double *du, const double *dv)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) return bad(c, "fvm_set_grid has not been called");
    int rc = fvm::setup_init(c, du, dv);
    if (rc == FVM_OK) c->init_done = true;
    return rc;
}

int fvm_upload_state(fvm_ctx *c, const double *u, const double *v, const double *p, const double *t,
                     const double *nlx, const double *nly, const double *adv)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) return bad(c, "fvm_set_grid has not been called");
    const size_t bytes = sizeof(double) * c->n;
    Dev &d = c->d;
    const double *src[] = {u, v, p, t, nlx, nly, adv};
    double *dst[] = {d.U, d.V, d.P, d.T, d.NLX, d.NLY, d.ADV};
    for (int k = 0; k < 7; k++)
        if (src[k]) FVM_CUDA(c, cudaMemcpyAsync(dst[k], src[k], bytes, cudaMemcpyHostToDevice, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    c->init_done = true;
    return FVM_OK;
}

int fvm_download_state(fvm_ctx *c, double *u, double *v, double *p, double *t, double *nlx, double *nly,
                       double *adv)
{
    if (!c) return FVM_ERR_ARG;
    const size_t bytes = sizeof(double) * c->n;
    Dev &d = c->d;
    double *dst[] = {u, v, p, t, nlx, nly, adv};
    const double *src[] = {d.U, d.V, d.P, d.T, d.NLX, d.NLY, d.ADV};
    for (int k = 0; k < 7; k++)
        if (dst[k]) FVM_CUDA(c, cudaMemcpyAsync(dst[k], src[k], bytes, cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

int fvm_get_array(fvm_ctx *c, const char *name, double *out)
{
    if (!c || !name || !out) return bad(c, "null argument");
    double *a = fvm::array_by_name(c, name);
    if (!a) return bad(c, "unknown array name");
    FVM_CUDA(c, cudaMemcpyAsync(out, a, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

int fvm_set_array(fvm_ctx *c, const char *name, const double *in)
{
    if (!c || !name || !in) return bad(c, "null argument");
    double *a = fvm::array_by_name(c, name);
    if (!a) return bad(c, "unknown array name");
    FVM_CUDA(c, cudaMemcpyAsync(a, in, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

int fvm_set_time(fvm_ctx *c, double rtime, int niter_time)
{
    if (!c) return FVM_ERR_ARG;
    c->rtime = rtime;
    c->niter_time = niter_time;
    return FVM_OK;
}

int fvm_adjoint_drag_grad(fvm_ctx *c, int window, int ckpt, double *J, double *dJ_domega, double *dJ_dblow)
{
    int r = need_ready(c);
    if (r) return r;
    if (window < 1 || ckpt < 1) return bad(c, "window and checkpoint interval must be positive");
    return fvm::run_adjoint(c, window, ckpt, J, dJ_domega, dJ_dblow);
}

int fvm_adjoint_vjp(fvm_ctx *c, double *lu, double *lv, double *lp, double *lnlx, double *lnly, double *dctrl)
{
    int r = need_ready(c);
    if (r) return r;
    if (!lu || !lv || !lp || !lnlx || !lnly) return bad(c, "null adjoint array");
    double *lam[5] = {lu, lv, lp, lnlx, lnly};
    return fvm::run_adjoint_vjp(c, lam, dctrl);
}

int fvm_set_controls(fvm_ctx *c, double omega, const double *blow)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) return bad(c, "fvm_set_controls needs the grid");
    if (!std::isfinite(omega)) return bad(c, "non-finite rotation rate");
    if (blow)
        for (int j = 0; j < c->NJ - 1; j++)
            if (!std::isfinite(blow[j])) return bad(c, "non-finite blowing speed");
    return fvm::setup_controls(c, omega, blow);
}

#define READY()                          \
    do {                                 \
        int r_ = need_ready(c);          \
        if (r_) return r_;               \
    } while (0)

int fvm_begin_step(fvm_ctx *c) { READY(); return fvm::run_begin_step(c); }
int fvm_contra_vel(fvm_ctx *c) { READY(); return fvm::run_contra_vel(c); }
int fvm_nl(fvm_ctx *c, int field)
{
    READY();
    if (field < FVM_FIELD_U || field > FVM_FIELD_T) return bad(c, "unknown field");
    return fvm::run_nl(c, field);
}
int fvm_dif(fvm_ctx *c, int field)
{
    READY();
    if (field < FVM_FIELD_U || field > FVM_FIELD_T) return bad(c, "unknown field");
    return fvm::run_dif(c, field);
}
int fvm_p_source(fvm_ctx *c) { READY(); return fvm::run_p_source(c); }
int fvm_iter_u(fvm_ctx *c) { READY(); return fvm::run_iter_u(c, FVM_FIELD_U); }
int fvm_iter_v(fvm_ctx *c) { READY(); return fvm::run_iter_u(c, FVM_FIELD_V); }
int fvm_remove_grad(fvm_ctx *c) { READY(); return fvm::run_remove_grad(c); }
int fvm_iter_p(fvm_ctx *c, double *resid, int *sweeps) { READY(); return fvm::run_iter_p(c, resid, sweeps); }
int fvm_correct(fvm_ctx *c) { READY(); return fvm::run_correct(c); }
int fvm_iter_t(fvm_ctx *c) { READY(); return fvm::run_iter_t(c); }
int fvm_calccoef(fvm_ctx *c, fvm_coeffs *out) { READY(); return fvm::run_calccoef(c, out); }

int fvm_step(fvm_ctx *c, int nsteps, fvm_coeffs *out)
{
    READY();
    if (nsteps < 0) return bad(c, "nsteps must be >= 0");
    return fvm::run_step(c, nsteps, out);
}

int fvm_history(fvm_ctx *c, fvm_coeffs *out, int n)
{
    if (!c || !out || n < 0) return FVM_ERR_ARG;
    int m = n < (int)c->hist.size() ? n : (int)c->hist.size();
    for (int k = 0; k < m; k++) out[k] = c->hist[k];
    return FVM_OK;
}

int fvm_synchronize(fvm_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

int fvm_get_stream(fvm_ctx *c, void **stream)
{
    if (!c || !stream) return FVM_ERR_ARG;
    *stream = (void *)c->stream;
    return FVM_OK;
}

int fvm_timing_reset(fvm_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    c->tm = fvm_timing{};
    return FVM_OK;
}

int fvm_time_sweeps(fvm_ctx *c, int sweeps, double *ms_per_launch, long long *launches)
{
    READY();
    if (sweeps < 1 || !ms_per_launch || !launches) return bad(c, "bad sweep timing arguments");
    return fvm::run_time_sweeps(c, sweeps, ms_per_launch, launches);
}

int fvm_get_timing(fvm_ctx *c, fvm_timing *out)
{
    if (!c || !out) return FVM_ERR_ARG;
    *out = c->tm;
    return FVM_OK;
}

int fvm_resident_wait_test(fvm_ctx *c, int max_polls)
{
    READY();
    if (max_polls < 1 || max_polls > (1 << 24)) return bad(c, "max_polls must be in 1 .. 2^24");
    return fvm::run_resident_wait_test(c, max_polls);
}

int fvm_resident_info(fvm_ctx *c, int *lines_per_block, int *blocks, int *sweeps_per_exchange)
{
    READY();
    if (!lines_per_block || !blocks || !sweeps_per_exchange) return bad(c, "null output pointer");
    *lines_per_block = c->res_lines;
    *blocks = c->res_blocks;
    *sweeps_per_exchange = c->res_lines ? c->res_depth : 0;
    return FVM_OK;
}

}  // extern "C"

namespace fvm {

double *array_by_name(fvm_ctx *c, const char *name)
{
    Dev &d = c->d;
    struct { const char *n; double *a; } t[] = {
        {"U", d.U}, {"V", d.V}, {"P", d.P}, {"T", d.T}, {"U_N", d.U_N}, {"V_N", d.V_N}, {"T_N", d.T_N},
        {"NLX", d.NLX}, {"NLY", d.NLY}, {"ADV", d.ADV}, {"NLX_NM1", d.NLX_NM1}, {"NLY_NM1", d.NLY_NM1},
        {"ADV_NM1", d.ADV_NM1}, {"DIFX", d.DIFX}, {"DIFY", d.DIFY}, {"DIFT", d.DIFT}, {"S_U", d.S_U},
        {"S_V", d.S_V}, {"UE", d.UE}, {"UW", d.UW}, {"VN", d.VN}, {"VS", d.VS}, {"X", d.X}, {"Y", d.Y},
        {"XG", d.XG}, {"YG", d.YG}, {"XIX", d.XIX}, {"XIY", d.XIY}, {"ETX", d.ETX}, {"ETY", d.ETY},
        {"DJAC", d.DJAC}, {"Q11", d.Q11}, {"Q12", d.Q12}, {"Q22", d.Q22}, {"DE", d.DE}, {"DW", d.DW},
        {"DN", d.DN}, {"DS", d.DS}, {"THETA", d.THETA}, {"AREA", d.AREA}, {"DIVDT", d.DIVDT},
        {"SU", d.SU}, {"SUV", d.SUV}, {"SUT", d.SUT}, {"DD", d.DD}};
    for (auto &e : t)
        if (std::strcmp(e.n, name) == 0) return e.a;
    return post_array(c, name);
}

}  // namespace fvm
