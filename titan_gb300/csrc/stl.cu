// stl.cu -- point-in-mesh classification for STL import (the GPU form of the
// reference's stl::stlFile::inside, include/Titan/stlparser.h:213-276, used by
// Simulation::importFromSTL, src/sim.cu:1855-1921).
//
// A point is inside when more than half of num_rays rays from it cross the
// triangle mesh an odd number of times.  Each ray direction is a vector of
// three uniform values in [-1000, 1000) divided by its norm, as the
// reference draws them -- but from a counter-based generator (SplitMix64 of
// seed, point index and ray index) instead of rand(), so that a
// classification is reproducible and identical on the GPU and in the CPU
// oracle.  Ray-triangle test: the reference's Moller-Trumbore form (edge
// vectors, cross and dot products in its operation order, epsilon 1e-6).
//
// One thread per point; triangles are staged through shared memory in
// chunks, and each thread keeps one parity bit per ray.
#include <cstdint>

#include <cuda_runtime.h>

#include "titan_gb300.h"

namespace {

constexpr int kStlThreads = 256;
constexpr int kStlChunk = 256;  // triangles per shared-memory chunk (9 doubles each)
constexpr int kStlMaxRays = 64;

__host__ __device__ inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

// uniform in [-1000, 1000): 53 random bits
__host__ __device__ inline double ray_component(uint64_t seed, int64_t point, int ray, int c) {
    const uint64_t k = splitmix64(seed ^ splitmix64((uint64_t)point * 3ULL * kStlMaxRays + (uint64_t)ray * 3ULL + c));
    const double u = (double)(k >> 11) * (1.0 / 9007199254740992.0);
    return -1000.0 + u * 2000.0;
}

__device__ inline double dot3(const double *a, const double *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

__device__ inline void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = b[0] * a[2] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// Moller-Trumbore with the reference's operation order (stlparser.h:213-246)
__device__ inline bool ray_hits(const double *p, const double *ray, const double *t) {
    const double eps = 0.000001;
    const double e1[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]};
    const double e2[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
    double h[3];
    cross3(ray, e2, h);
    const double a = dot3(e1, h);
    if (a > -eps && a < eps) return false;
    const double f = 1 / a;
    const double s[3] = {p[0] - t[0], p[1] - t[1], p[2] - t[2]};
    const double u = f * dot3(s, h);
    if (u < 0 || u > 1.0) return false;
    double q[3];
    cross3(s, e1, q);
    const double v = f * dot3(ray, q);
    if (v < 0 || u + v > 1.0) return false;
    return f * dot3(e2, q) > eps;
}

__global__ void __launch_bounds__(kStlThreads) k_stl_inside(const double *tri, int64_t ntri, const double *pts,
                                                              int64_t npts, int num_rays, uint64_t seed,
                                                              uint8_t *inside) {
    __shared__ double st[kStlChunk * 9];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < npts;
    double p[3] = {0, 0, 0};
    if (live)
        for (int c = 0; c < 3; c++) p[c] = pts[3 * i + c];
    double rays[kStlMaxRays][3];  // the thread's ray directions (local memory)
    for (int r = 0; r < num_rays; r++) {
        double d[3];
        for (int c = 0; c < 3; c++) d[c] = ray_component(seed, i, r, c);
        const double n = sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
        for (int c = 0; c < 3; c++) rays[r][c] = d[c] / n;
    }
    uint64_t parity = 0;
    for (int64_t t0 = 0; t0 < ntri; t0 += kStlChunk) {
        const int nt = (int)(ntri - t0 < kStlChunk ? ntri - t0 : kStlChunk);
        __syncthreads();
        for (int q = threadIdx.x; q < nt * 9; q += blockDim.x) st[q] = tri[t0 * 9 + q];
        __syncthreads();
        if (!live) continue;
        for (int r = 0; r < num_rays; r++) {
            const double rr[3] = {rays[r][0], rays[r][1], rays[r][2]};
            uint64_t b = 0;
            for (int t = 0; t < nt; t++) b ^= (uint64_t)ray_hits(p, rr, st + 9 * t);
            parity ^= b << r;
        }
    }
    if (live) {
        const int odd = __popcll(parity);
        inside[i] = (double)odd / (double)num_rays > 0.5 ? 1 : 0;
    }
}

}  // namespace

extern "C" int titan_gb300_stl_inside(int device, const double *tri, int64_t ntri, const double *pts, int64_t npts,
                                      int num_rays, uint64_t seed, uint8_t *inside) {
    if (!tri || !pts || !inside || ntri < 0 || npts < 0 || num_rays < 1 || num_rays > kStlMaxRays)
        return TITAN_GB300_EINVAL;
    if (npts == 0) return TITAN_GB300_OK;
    if (cudaSetDevice(device) != cudaSuccess) return TITAN_GB300_ECUDA;
    double *d_tri = nullptr, *d_pts = nullptr;
    uint8_t *d_in = nullptr;
    cudaStream_t s = nullptr;
    int rc = TITAN_GB300_OK;
    do {
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { rc = TITAN_GB300_ECUDA; break; }
        if (cudaMalloc(&d_tri, (size_t)(ntri > 0 ? ntri : 1) * 9 * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&d_pts, (size_t)npts * 3 * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&d_in, (size_t)npts) != cudaSuccess) {
            rc = TITAN_GB300_ENOMEM;
            break;
        }
        if (ntri > 0 &&
            cudaMemcpyAsync(d_tri, tri, (size_t)ntri * 9 * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess) {
            rc = TITAN_GB300_ECUDA;
            break;
        }
        if (cudaMemcpyAsync(d_pts, pts, (size_t)npts * 3 * sizeof(double), cudaMemcpyHostToDevice, s) !=
            cudaSuccess) {
            rc = TITAN_GB300_ECUDA;
            break;
        }
        const unsigned blocks = (unsigned)((npts + kStlThreads - 1) / kStlThreads);
        k_stl_inside<<<blocks, kStlThreads, 0, s>>>(d_tri, ntri, d_pts, npts, num_rays, seed, d_in);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(inside, d_in, (size_t)npts, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            rc = TITAN_GB300_ECUDA;
    } while (false);
    cudaFree(d_tri);
    cudaFree(d_pts);
    cudaFree(d_in);
    if (s) cudaStreamDestroy(s);
    return rc;
}
