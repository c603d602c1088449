// fvm_post.cu -- the post-processing phase of the 2-D solver: CALC_VOR
// (calc_vor.f90:14-58), the post-processing block of CALCCOEF
// (calccoef.f90:156-190) and POST_PROCESS (post_process.f90:8-62).
//
// The field work (vorticity and the time sums of U, V, P, T, VOR) is one kernel
// over the whole (0:NI, 0:NJ) array; the branch-cut rows J=0 and J=NJ, which the
// reference copies from J=NJ-1 and J=1, are evaluated there directly, so no
// second pass is needed.  The scalar bookkeeping (lift extrema, Strouhal number,
// sums and rms) works on the coefficient record that CALCCOEF has already copied
// to the host, in the reference's order of operations.
#include <cmath>
#include <cstring>

#include "fvm_internal.cuh"

namespace fvm {
namespace {

// Vorticity of cell (i, j), 1 <= j <= NJ-1, 0 <= i <= NI: centred differences in
// the interior, the extrapolated ghost value 3q(0)-3q(1)+q(2) (and its mirror at
// I=NI) in the I difference of the boundary rows.
__device__ __forceinline__ double vor_at(const Dev &d, int i, int j)
{
    const double *U = d.U, *V = d.V;
    const int c = IDX(i, j);
    double dv, du;
    if (i == 0) {
        dv = V[IDX(1, j)] - ((3.0 * V[c] - 3.0 * V[IDX(1, j)]) + V[IDX(2, j)]);
        du = U[IDX(1, j)] - ((3.0 * U[c] - 3.0 * U[IDX(1, j)]) + U[IDX(2, j)]);
    } else if (i == d.NI) {
        dv = ((3.0 * V[c] - 3.0 * V[IDX(i - 1, j)]) + V[IDX(i - 2, j)]) - V[IDX(i - 1, j)];
        du = ((3.0 * U[c] - 3.0 * U[IDX(i - 1, j)]) + U[IDX(i - 2, j)]) - U[IDX(i - 1, j)];
    } else {
        dv = V[IDX(i + 1, j)] - V[IDX(i - 1, j)];
        du = U[IDX(i + 1, j)] - U[IDX(i - 1, j)];
    }
    return (((d.XIX[c] * 0.5) * dv + (d.ETX[c] * 0.5) * (V[IDX(i, j + 1)] - V[IDX(i, j - 1)])) -
            (d.XIY[c] * 0.5) * du) -
           (d.ETY[c] * 0.5) * (U[IDX(i, j + 1)] - U[IDX(i, j - 1)]);
}

// arr: VOR, U_TA, V_TA, P_TA, T_TA, VOR_TA (n each).  accumulate = 0: CALC_VOR only.
__global__ void k_post(const Dev d, double *arr, int accumulate)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n) return;
    const int i = c % d.NI1, j = c / d.NI1;
    const int jj = j == 0 ? d.NJ - 1 : (j == d.NJ ? 1 : j);   // calc_vor.f90:46-57
    const double w = vor_at(d, i, jj);
    const size_t n = d.n;
    arr[c] = w;
    if (!accumulate) return;
    arr[n + c] += d.U[c];
    arr[2 * n + c] += d.V[c];
    arr[3 * n + c] += d.P[c];
    arr[4 * n + c] += d.T[c];
    arr[5 * n + c] += w;
}

int post_alloc(fvm_ctx *c)
{
    if (c->post.arr) return FVM_OK;
    FVM_CUDA(c, cudaMalloc(&c->post.arr, sizeof(double) * 6 * size_t(c->n)));
    FVM_CUDA(c, cudaMemsetAsync(c->post.arr, 0, sizeof(double) * 6 * size_t(c->n), c->stream));
    return FVM_OK;
}

int launch_post(fvm_ctx *c, int accumulate)
{
    k_post<<<(c->n + 255) / 256, 256, 0, c->stream>>>(c->d, c->post.arr, accumulate);
    KCOUNT(c);
    FVM_LAUNCH_CHECK(c);
    return FVM_OK;
}

}  // namespace

int post_after_calccoef(fvm_ctx *c, double cl_prev, const fvm_coeffs &co)
{
    PostState &s = c->post;
    if (!s.ipost || c->post_suspend) return FVM_OK;
    int rc = launch_post(c, 1);   // CALC_VOR and the field sums
    if (rc) return rc;
    s.niter_pos = s.niter_pos + 1;
    const double cl = co.cl, rtime = co.time;
    if ((double)s.toggle * (cl - cl_prev) < 0.0) {   // an extremum of the lift: half a period
        s.toggle = -1 * s.toggle;
        s.st = 1.0 / (rtime - s.time2);
        s.time2 = s.time1;
        s.time1 = rtime;
        s.cl_amp = std::fabs(cl - s.cl1) / 2.0;
        s.cl1 = cl;
    }
    s.nu_ta = s.nu_ta + co.nu;
    s.cd_ta = s.cd_ta + co.cd;
    s.cl_ta = s.cl_ta + cl;
    s.st_ta = s.st_ta + s.st;
    s.cpb_ta = s.cpb_ta + co.cpb;
    s.cl_amp_ta = s.cl_amp_ta + s.cl_amp;
    const double n = (double)s.niter_pos;
    const double dum_a = s.cd_ta / n, dum_b = s.cl_ta / n;
    s.rms_cd = s.rms_cd + (co.cd - dum_a) * (co.cd - dum_a);
    s.rms_cl = s.rms_cl + (cl - dum_b) * (cl - dum_b);
    fvm_post &r = s.rec;
    r.time = rtime;
    r.nu = s.nu_ta / n;
    r.cd = dum_a;
    r.cl = dum_b;
    r.cl_amp = s.cl_amp_ta / n;
    r.cpb = s.cpb_ta / n;
    r.st = s.st_ta / n;
    r.rms_cd = std::sqrt(s.rms_cd / n);
    r.rms_cl = std::sqrt(s.rms_cl / n);
    r.st_last = s.st;
    r.cl_amp_last = s.cl_amp;
    r.niter = s.niter_pos;
    return FVM_OK;
}

void post_free(fvm_ctx *c)
{
    if (c->post.arr) cudaFree(c->post.arr);
    c->post.arr = nullptr;
}

double *post_array(fvm_ctx *c, const char *name)
{
    if (!c->post.arr) return nullptr;
    const char *names[] = {"VOR", "U_TA", "V_TA", "P_TA", "T_TA", "VOR_TA"};
    for (int q = 0; q < 6; q++)
        if (std::strcmp(names[q], name) == 0) return c->post.arr + size_t(q) * c->n;
    return nullptr;
}

}  // namespace fvm

extern "C" {

int fvm_post_begin(fvm_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->grid_set) {
        c->err = "fvm_set_grid has not been called";
        return FVM_ERR_ARG;
    }
    int rc = fvm::post_alloc(c);
    if (rc) return rc;
    fvm::PostState &s = c->post;
    // post_process.f90:8-16; ST, CL_AMP, CL1, TIME1, TIME2 keep their values
    s.niter_pos = 0;
    s.toggle = 1;
    s.ipost = 1;
    s.nu_ta = s.cd_ta = s.cl_ta = s.st_ta = s.cpb_ta = s.cl_amp_ta = 0.0;
    s.rms_cd = s.rms_cl = 0.0;
    s.rec = fvm_post{};
    FVM_CUDA(c, cudaMemsetAsync(s.arr + c->n, 0, sizeof(double) * 5 * size_t(c->n), c->stream));
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

int fvm_post_get(fvm_ctx *c, fvm_post *out)
{
    if (!c || !out) return FVM_ERR_ARG;
    *out = c->post.rec;
    return FVM_OK;
}

int fvm_post_final(fvm_ctx *c, fvm_post *out, double *u, double *v, double *p, double *t, double *vor)
{
    if (!c) return FVM_ERR_ARG;
    const fvm::PostState &s = c->post;
    if (!s.arr || s.niter_pos < 1) {
        c->err = "no post-processing steps have been averaged";
        return FVM_ERR_ARG;
    }
    const double n = (double)s.niter_pos;
    double *dst[5] = {u, v, p, t, vor};
    for (int q = 0; q < 5; q++) {   // post_process.f90:22-26
        if (!dst[q]) continue;
        FVM_CUDA(c, cudaMemcpyAsync(dst[q], s.arr + size_t(q + 1) * c->n, sizeof(double) * c->n,
                                    cudaMemcpyDeviceToHost, c->stream));
    }
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int q = 0; q < 5; q++)
        if (dst[q])
            for (int e = 0; e < c->n; e++) dst[q][e] = dst[q][e] / n;
    if (out) {   // post_process.f90:27-36
        out->time = c->rtime;
        out->nu = s.nu_ta / n;
        out->cd = s.cd_ta / n;
        out->cl = s.cl_ta / n;
        out->st = s.st_ta / n;
        out->cpb = s.cpb_ta / n;
        out->cl_amp = s.cl_amp_ta / n;
        out->rms_cd = std::sqrt(s.rms_cd / n);
        out->rms_cl = std::sqrt(s.rms_cl / n);
        out->st_last = s.st;
        out->cl_amp_last = s.cl_amp;
        out->niter = s.niter_pos;
    }
    return FVM_OK;
}

int fvm_post_end(fvm_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    c->post.ipost = 0;
    return FVM_OK;
}

int fvm_calc_vor(fvm_ctx *c)
{
    if (!c) return FVM_ERR_ARG;
    if (!c->init_done) {
        c->err = "fvm_init has not been called";
        return FVM_ERR_ARG;
    }
    int rc = fvm::post_alloc(c);
    if (rc) return rc;
    rc = fvm::launch_post(c, 0);
    if (rc) return rc;
    FVM_CUDA(c, cudaStreamSynchronize(c->stream));
    return FVM_OK;
}

}  // extern "C"
