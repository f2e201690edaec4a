// noalloc.cu -- energy and momentum diagnostics that allocate nothing.
//
// Some callers cannot call cudaMalloc at the moment they need a result: a
// real-time control loop that may only use memory reserved at start-up, a
// host framework whose caching allocator owns all device memory, or code
// that runs while a CUDA stream is being captured into a graph.  For them,
// titan_gb300_diagnostics_noalloc computes the same FP64 quantities as
// titan_gb300_diagnostics from state the caller already holds in device
// memory, using as scratch a fixed array compiled into this library.
//
// The scratch array (kNoAllocBlocks x 9 doubles, 288 KiB) is a file-scope
// __device__ variable: every GPU that loads the library holds it until the
// process exits.  Host code cannot use its name as a device address; the
// address comes from cudaGetSymbolAddress, looked up once per device on the
// first call made on that device (so that first call should be made before
// any stream capture starts).  Every call shares the array and overwrites
// the slots it uses; two calls that overlap on the GPU (for instance on two
// streams) race on it and must be ordered by the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "titan_gb300.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocItems = 64;        // elements per thread per pass
constexpr int kNoAllocBlocks = 4096;     // partial-sum slots in the scratch
constexpr int kNoAllocQ = 9;             // spring PE, KE, gravity PE, p(3), L(3)
constexpr int64_t kNoAllocMaxElems = (int64_t)kNoAllocBlocks * kNoAllocThreads * kNoAllocItems;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocBlocks * kNoAllocQ];

std::mutex g_setup_mu;
double *g_scratch_ptr[256] = {nullptr};

__device__ __forceinline__ double nrm3(double a, double b, double c) { return sqrt((a * a + b * b) + c * c); }

// One thread sums kNoAllocItems strided masses and springs of its block's
// range; the block reduces with a fixed tree and writes one partial slot.
__global__ void __launch_bounds__(kNoAllocThreads)
k_noalloc_diag1(const double *pos, const double *vel, const double *m, int64_t n, const int32_t *left,
                const int32_t *right, const double *k, const double *rest, int64_t ns, double g_mag,
                double *scratch) {
    __shared__ double red[kNoAllocQ][kNoAllocThreads];
    double q[kNoAllocQ];
#pragma unroll
    for (int c = 0; c < kNoAllocQ; c++) q[c] = 0.0;
    const int64_t base = (int64_t)blockIdx.x * kNoAllocThreads * kNoAllocItems + threadIdx.x;
    for (int it = 0; it < kNoAllocItems; it++) {
        const int64_t i = base + (int64_t)it * kNoAllocThreads;
        if (i < n) {
            const double mm = m[i];
            const double x0 = pos[3 * i], x1 = pos[3 * i + 1], x2 = pos[3 * i + 2];
            const double v0 = vel[3 * i], v1 = vel[3 * i + 1], v2 = vel[3 * i + 2];
            const double vn = nrm3(v0, v1, v2);
            q[1] += (0.5 * mm) * (vn * vn);
            q[2] += (g_mag * x2) * mm;
            const double p0 = v0 * mm, p1 = v1 * mm, p2 = v2 * mm;
            q[3] += p0;
            q[4] += p1;
            q[5] += p2;
            q[6] += p1 * x2 - p2 * x1;
            q[7] += x0 * p2 - p0 * x2;
            q[8] += p0 * x1 - p1 * x0;
        }
        if (i < ns) {
            const int32_t l = left[i], r = right[i];
            if (l >= 0 && r >= 0 && l < n && r < n) {
                const double d0 = pos[3 * l] - pos[3 * r], d1 = pos[3 * l + 1] - pos[3 * r + 1],
                             d2 = pos[3 * l + 2] - pos[3 * r + 2];
                const double x = nrm3(d0, d1, d2) - rest[i];
                q[0] += (k[i] * (x * x)) / 2;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kNoAllocQ; c++) red[c][threadIdx.x] = q[c];
    __syncthreads();
    for (int w = kNoAllocThreads / 2; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int c = 0; c < kNoAllocQ; c++) red[c][threadIdx.x] += red[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kNoAllocQ) scratch[blockIdx.x * kNoAllocQ + threadIdx.x] = red[threadIdx.x][0];
}

// Reduces the nblocks partial slots written by this call into out[9].
__global__ void __launch_bounds__(kNoAllocThreads)
k_noalloc_diag2(const double *scratch, int nblocks, double *out) {
    __shared__ double red[kNoAllocQ][kNoAllocThreads];
    for (int c = 0; c < kNoAllocQ; c++) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += kNoAllocThreads) s += scratch[b * kNoAllocQ + c];
        red[c][threadIdx.x] = s;
    }
    __syncthreads();
    for (int w = kNoAllocThreads / 2; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int c = 0; c < kNoAllocQ; c++) red[c][threadIdx.x] += red[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kNoAllocQ) out[threadIdx.x] = red[threadIdx.x][0];
}

// Device address of the scratch array on the current device, looked up once.
cudaError_t scratch_for_current_device(double **ptr) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *ptr = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int titan_gb300_diagnostics_noalloc(const double *pos, const double *vel, const double *m, int64_t n,
                                               const int32_t *left, const int32_t *right, const double *k,
                                               const double *rest, int64_t ns, double g_mag, double *out,
                                               void *stream) {
    if (n < 0 || ns < 0 || !out) return TITAN_GB300_EINVAL;
    if (n > 0 && (!pos || !vel || !m)) return TITAN_GB300_EINVAL;
    if (ns > 0 && (!left || !right || !k || !rest)) return TITAN_GB300_EINVAL;
    if (n > kNoAllocMaxElems || ns > kNoAllocMaxElems) return TITAN_GB300_ELIMIT;
    double *scratch = nullptr;
    if (scratch_for_current_device(&scratch) != cudaSuccess) return TITAN_GB300_ECUDA;
    const int64_t work = n > ns ? n : ns;
    const int64_t per_block = (int64_t)kNoAllocThreads * kNoAllocItems;
    int nblocks = (int)((work + per_block - 1) / per_block);
    if (nblocks < 1) nblocks = 1;
    cudaStream_t st = (cudaStream_t)stream;
    k_noalloc_diag1<<<nblocks, kNoAllocThreads, 0, st>>>(pos, vel, m, n, left, right, k, rest, ns, g_mag, scratch);
    if (cudaGetLastError() != cudaSuccess) return TITAN_GB300_ECUDA;
    k_noalloc_diag2<<<1, kNoAllocThreads, 0, st>>>(scratch, nblocks, out);
    if (cudaGetLastError() != cudaSuccess) return TITAN_GB300_ECUDA;
    return TITAN_GB300_OK;
}
