// lpm_update_rr_noalloc: the residual update of one Newton iteration (updateRR
// plus the two norms the Newton test reads) on caller-owned device arrays,
// without allocating device memory.
//
// Who needs it: callers that cannot call cudaMalloc, for example a host code
// whose device memory is handed out by its own pool or a fixed budget (the
// application owns every byte and forbids a library from growing the
// footprint), or code running where allocation is not allowed.  They pass
// their own input and output arrays; the only work space is the fixed
// file-scope device array below (its size is set at compile time and every
// GPU that loads this library holds it until the process exits).
//
// The array is shared by every call on a device and keeps the contents of the
// last call.  Calls whose kernels overlap on the GPU (different streams or
// host threads without ordering between them) race on it and give wrong
// norms; order such calls on one stream or synchronise between them.
#include <cmath>
#include <mutex>
#include <string>
#include "lpm_internal.h"

namespace lpm {
namespace {

constexpr int RR_TPB = 256;
constexpr int RR_MAX_BLOCKS = LPM_NOALLOC_MAX_PARTICLES / RR_TPB;
// scratch layout in doubles: [0, 2*RR_MAX_BLOCKS) per-block partial sums
// (|residual|^2, |reaction|^2), then the two totals, then the last-block
// counter (an unsigned in the first word of its slot)
constexpr int RR_NORMS = 2 * RR_MAX_BLOCKS;
constexpr int RR_COUNTER = RR_NORMS + 2;
constexpr int RR_SCRATCH_DOUBLES = RR_COUNTER + 2;

static_assert(LPM_NOALLOC_MAX_PARTICLES % RR_TPB == 0, "limit must be a whole number of blocks");

// The scratch array (256 KB + 32 B).  In host code this name is a host-side
// stand-in, not a device address: the kernel gets the device address from
// cudaGetSymbolAddress, once per device (rr_scratch_of below).
static __device__ __align__(256) double g_rr_scratch[RR_SCRATCH_DOUBLES];

constexpr int RR_MAX_DEVICES = 64;
std::mutex g_rr_mutex;
double *g_rr_ptr[RR_MAX_DEVICES] = {nullptr};

// updateRR (src/stiffness.c:519-534) for particle i, in the reference's
// layout (3 DOFs per particle, dispBC_index 1 = free, 0 = prescribed), and
// the squared norms of the residual and of the reaction forces (Pin on the
// prescribed DOFs: the list cblas_dnrm2 reads at src/lpmc_project.c:412-413).
// Deterministic: block tree sums, then the last block adds the partials in
// block order.
__global__ void __launch_bounds__(RR_TPB) k_update_rr_noalloc(int n, const double *__restrict__ Pin,
                                                              const double *__restrict__ Pex,
                                                              const int *__restrict__ bc,
                                                              double *__restrict__ res, double *scratch)
{
    __shared__ double red[2][RR_TPB / 32];
    __shared__ bool last;
    const int i = blockIdx.x * RR_TPB + threadIdx.x;
    double v0 = 0.0, v1 = 0.0;
    if (i < n) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const size_t d = 3 * (size_t)i + k;
            const double pin = Pin[d];
            const int m = bc[d];
            const double r = (double)m * (Pex[d] - pin);
            res[d] = r;
            v0 += r * r;
            if (m == 0)
                v1 += pin * pin;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_xor_sync(0xffffffffu, v0, o);
        v1 += __shfl_xor_sync(0xffffffffu, v1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = v0;
        red[1][threadIdx.x >> 5] = v1;
    }
    __syncthreads();
    unsigned *counter = reinterpret_cast<unsigned *>(scratch + RR_COUNTER);
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int w = 0; w < RR_TPB / 32; w++) {
            s0 += red[0][w];
            s1 += red[1][w];
        }
        scratch[2 * blockIdx.x] = s0;
        scratch[2 * blockIdx.x + 1] = s1;
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last)
        return;
    __threadfence();
    // the last block: thread t sums the partials t, t + RR_TPB, ... in order
    double s0 = 0.0, s1 = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RR_TPB) {
        s0 += __ldcg(&scratch[2 * b]);
        s1 += __ldcg(&scratch[2 * b + 1]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s0;
        red[1][threadIdx.x >> 5] = s1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int w = 0; w < RR_TPB / 32; w++) {
            t0 += red[0][w];
            t1 += red[1][w];
        }
        scratch[RR_NORMS] = t0;
        scratch[RR_NORMS + 1] = t1;
        *counter = 0u;
    }
}

// Device address of the scratch array on the current device.  The first call
// on a device looks it up (cudaGetSymbolAddress, which may load this
// library's kernels onto that device); later calls reuse the cached address.
// A device reset unloads the module and may reload it elsewhere, which is
// why the header rules out calls after one.
int rr_scratch_of(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return fail(LPM_ERR_CUDA, std::string("lpm_update_rr_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= RR_MAX_DEVICES)
        return fail(LPM_ERR_ARG, "lpm_update_rr_noalloc: device ordinal " + std::to_string(dev) +
                                     " beyond the " + std::to_string(RR_MAX_DEVICES) + " devices it serves");
    std::lock_guard<std::mutex> lock(g_rr_mutex);
    if (!g_rr_ptr[dev]) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_rr_scratch);
        if (e != cudaSuccess)
            return fail(LPM_ERR_CUDA,
                        std::string("lpm_update_rr_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_rr_ptr[dev] = p;
    }
    *out = g_rr_ptr[dev];
    return LPM_OK;
}

}  // namespace
}  // namespace lpm

extern "C" int lpm_update_rr_noalloc(int n, const double *Pin, const double *Pex, const int *dispBC_index,
                                     double *residual, double norms[2], void *stream)
{
    using namespace lpm;
    if (n < 0)
        return fail(LPM_ERR_ARG, "lpm_update_rr_noalloc: negative particle count");
    if (n > LPM_NOALLOC_MAX_PARTICLES)
        return fail(LPM_ERR_ARG, "lpm_update_rr_noalloc: " + std::to_string(n) +
                                     " particles exceed the fixed scratch limit of " +
                                     std::to_string(LPM_NOALLOC_MAX_PARTICLES) +
                                     " (LPM_NOALLOC_MAX_PARTICLES); use lpm_compute_force on a context");
    if (n > 0 && (!Pin || !Pex || !dispBC_index || !residual))
        return fail(LPM_ERR_ARG, "lpm_update_rr_noalloc: null array");
    if (n == 0) {
        if (norms)
            norms[0] = norms[1] = 0.0;
        return LPM_OK;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (norms) {
        // reading the norms waits on the stream, which a capture cannot hold
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaError_t ce = cudaStreamIsCapturing(s, &cs);
        if (ce != cudaSuccess)
            return fail(LPM_ERR_CUDA, std::string("lpm_update_rr_noalloc: cudaStreamIsCapturing: ") +
                                          cudaGetErrorString(ce));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(LPM_ERR_ARG, "lpm_update_rr_noalloc: norms must be NULL on a stream being captured");
    }
    double *scratch = nullptr;
    int rc = rr_scratch_of(&scratch);
    if (rc)
        return rc;
    // the last-block counter must start at zero (a call cut short could leave it set)
    cudaError_t e = cudaMemsetAsync(scratch + RR_COUNTER, 0, sizeof(unsigned), s);
    if (e != cudaSuccess)
        return fail(LPM_ERR_CUDA, std::string("lpm_update_rr_noalloc: cudaMemsetAsync: ") + cudaGetErrorString(e));
    const int blocks = (n + RR_TPB - 1) / RR_TPB;
    k_update_rr_noalloc<<<blocks, RR_TPB, 0, s>>>(n, Pin, Pex, dispBC_index, residual, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return fail(LPM_ERR_CUDA, std::string("lpm_update_rr_noalloc: launch: ") + cudaGetErrorString(e));
    if (!norms)
        return LPM_OK;
    double h[2] = {0.0, 0.0};
    e = cudaMemcpyAsync(h, scratch + RR_NORMS, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return fail(LPM_ERR_CUDA, std::string("lpm_update_rr_noalloc: reading the norms: ") + cudaGetErrorString(e));
    norms[0] = std::sqrt(h[0]);
    norms[1] = std::sqrt(h[1]);
    return LPM_OK;
}
