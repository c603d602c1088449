// fvm_static.cu -- allocation-free variant of the pressure-residual kernel.
//
// Who needs it: a caller that owns its device arrays but may not allocate device
// memory itself -- code running while a CUDA stream is being captured into a graph
// (cudaMalloc is not permitted during capture), a host program whose device memory
// comes from a pool or a framework allocator it does not control, or a Fortran
// driver that only hands over pre-allocated buffers.  fvm_poisson_residual_static
// needs no context and calls no allocating routine: its only scratch (the per-block
// partial sums and the arrival ticket of the two-level reduction) is the static
// device array below, resolved once per device with cudaGetSymbolAddress.
#include <mutex>

#include "fvm_internal.cuh"
#include "fvm_ops.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 2;
constexpr int kMaxBlocks = 2048;
// Largest interior grid accepted: 2048 blocks x 256 threads x 2 cells.
constexpr long long kMaxCells = (long long)kMaxBlocks * kThreads * kCellsPerThread;
// Words 0 .. 2*kMaxBlocks-1 hold the block partial sums; word 2*kMaxBlocks holds
// the arrival ticket (cleared at every call).  32 KiB + 256 B per device.
constexpr int kScratchWords = 2 * kMaxBlocks + 32;

static __device__ __align__(256) double g_resid_scratch[kScratchWords];

// Scaled L1 residual sum|r| / sum|AP*P| over the interior (iter_p.f90:37-50),
// r = AE P(i+1) + AW P(i-1) + AN P(j+1) + AS P(j-1) + SU - AP P with the
// circumferential neighbours read through periodic wrap.
__global__ void __launch_bounds__(kThreads) k_resid_static(int NI, int NJ, const double *P, const double *SU,
                                                           const double *AP, const double *AE, const double *AW,
                                                           const double *AN, const double *AS, double *scratch,
                                                           double *out)
{
    __shared__ double sh[64];
    __shared__ bool last;
    const int NI1 = NI + 1, ni1 = NI - 1, total = ni1 * (NJ - 1);
    auto id = [&](int i, int j) { return i + NI1 * j; };
    double ra = 0.0, pa = 0.0;
#pragma unroll
    for (int q = 0; q < kCellsPerThread; q++) {
        int e = (blockIdx.x * kCellsPerThread + q) * kThreads + threadIdx.x;
        if (e < total) {
            int i = e % ni1 + 1, j = e / ni1 + 1, c = id(i, j);
            int jn = (j == NJ - 1) ? 1 : j + 1, js = (j == 1) ? NJ - 1 : j - 1;
            double p = P[c];
            double r = ((((AE[c] * P[id(i + 1, j)] + AW[c] * P[id(i - 1, j)]) + AN[c] * P[id(i, jn)])
                         + AS[c] * P[id(i, js)]) + SU[c]) - AP[c] * p;
            ra += fabs(r);
            pa += fabs(AP[c] * p);
        }
    }
    fvm::block_sum2(ra, pa, sh);
    unsigned int *ticket = reinterpret_cast<unsigned int *>(scratch + 2 * kMaxBlocks);
    if (threadIdx.x == 0) {
        scratch[2 * blockIdx.x] = ra;
        scratch[2 * blockIdx.x + 1] = pa;
        __threadfence();
        unsigned t = atomicInc(ticket, gridDim.x - 1);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
        a += ((volatile double *)scratch)[2 * k];
        b += ((volatile double *)scratch)[2 * k + 1];
    }
    fvm::block_sum2(a, b, sh);
    if (threadIdx.x == 0) *out = a / b;
}

std::mutex g_mu;
void *g_addr[64] = {};

// Device address of the static scratch on the current device (set up once per
// device, with that device current).  The address is kept for the life of the
// process: a cudaDeviceReset (or any other teardown of the device's primary
// context) unmaps it, so the library must not be used across a device reset.
cudaError_t scratch_address(int dev, double **ptr)
{
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_resid_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = p;
    }
    *ptr = static_cast<double *>(g_addr[dev]);
    return cudaSuccess;
}

}  // namespace

extern "C" int fvm_poisson_residual_static(int ni, int nj, const double *p, const double *su, const double *ap,
                                           const double *ae, const double *aw, const double *an,
                                           const double *as, double *resid, void *stream)
{
    // sizes first: an oversized grid is refused before any pointer is looked at
    if (ni < 3 || nj < 3) return FVM_ERR_ARG;
    const long long cells = (long long)(ni - 1) * (nj - 1);
    if (cells > kMaxCells) return FVM_ERR_ARG;
    if (!p || !su || !ap || !ae || !aw || !an || !as || !resid) return FVM_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FVM_ERR_CUDA;
    double *scratch = nullptr;
    if (scratch_address(dev, &scratch) != cudaSuccess) return FVM_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(scratch + 2 * kMaxBlocks, 0, sizeof(unsigned int), st) != cudaSuccess) return FVM_ERR_CUDA;
    const int blocks = (int)((cells + (long long)kThreads * kCellsPerThread - 1) / ((long long)kThreads * kCellsPerThread));
    k_resid_static<<<blocks, kThreads, 0, st>>>(ni, nj, p, su, ap, ae, aw, an, as, scratch, resid);
    if (cudaGetLastError() != cudaSuccess) return FVM_ERR_CUDA;
    return FVM_OK;
}
