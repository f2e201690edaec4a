// xfer.cu -- per-mass transfer between caller order and tiled order
// (get/set/getAll/setAll: src/sim.cu:588-764 in the reference) and the FP64
// energy / momentum diagnostics (test/testutil/utils.h:12-43).
#include <cstdint>

#include "engine.h"
#include "state.cuh"
#include "step_math.cuh"

namespace tg {

namespace {

// ------------------------------------------------- gather / scatter -------
template <int PREC>
__global__ void k_gather(XferArgs a) {
    using R = typename Real<PREC>::T;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    int64_t src = a.idx ? a.idx[i] : i;
    int64_t g = a.old2new[src];
    const St<PREC> s = load_state<PREC>(a.parity ? a.state1 : a.state0, g);
    const int64_t np = a.npad;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double x = (double)s.x[c], v = (double)s.v[c];
        if constexpr (PREC == P_FP32C) {
            x += (double)s.xl[c];
            v += (double)s.vl[c];
        }
        if (a.pos) a.pos[3 * i + c] = x;
        if (a.vel) a.vel[3 * i + c] = v;
        if (a.accout) a.accout[3 * i + c] = (double)reinterpret_cast<const R *>(a.acc)[c * np + g];
    }
}

// Positions of all masses in caller (creation) order as float triples, the
// headless form of the reference's updateVertices (src/sim.cu:1717-1725):
// (float) of the position (FP32C: of hi + lo in double).
template <int PREC>
__global__ void k_export_f32(XferArgs a, float *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    const int64_t g = a.old2new[i];
    const St<PREC> s = load_state<PREC>(a.parity ? a.state1 : a.state0, g);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double x = (double)s.x[c];
        if constexpr (PREC == P_FP32C) x += (double)s.xl[c];
        out[3 * i + c] = (float)x;
    }
}

// Writes pos and/or vel of the listed masses into both buffers, keeping the
// other field from the current buffer.
template <int PREC>
__global__ void k_scatter(XferArgs a) {
    using R = typename Real<PREC>::T;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    int64_t src = a.idx ? a.idx[i] : i;
    int64_t g = a.old2new[src];
    const int64_t np = a.npad;
    St<PREC> s = load_state<PREC>(a.parity ? a.state1 : a.state0, g);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (a.ipos) {
            double x = a.ipos[3 * i + c];
            s.x[c] = (R)x;
            if constexpr (PREC == P_FP32C) s.xl[c] = (R)(x - (double)s.x[c]);
        }
        if (a.ivel) {
            double v = a.ivel[3 * i + c];
            s.v[c] = (R)v;
            if constexpr (PREC == P_FP32C) s.vl[c] = (R)(v - (double)s.v[c]);
        }
        if (a.ipos) reinterpret_cast<R *>(a.acc)[c * np + g] = (R)0;
    }
    store_state<PREC>(a.state0, g, s);
    store_state<PREC>(a.state1, g, s);
}

// ------------------------------------------------------ diagnostics -------
// Pass 1: each of kDiagBlocks blocks sums a fixed grid-stride share in FP64
// and reduces it with a fixed tree; pass 2 reduces the partials the same way.
template <int PREC>
__global__ void __launch_bounds__(256) k_diag1(DiagArgs a) {
    __shared__ double red[kDiagQ][256];
    double q[kDiagQ];
#pragma unroll
    for (int k = 0; k < kDiagQ; k++) q[k] = 0.0;
    using R = typename Real<PREC>::T;
    const R *ms = reinterpret_cast<const R *>(a.mass);
    auto pos = [&](const St<PREC> &s, int c) {
        double x = (double)s.x[c];
        if constexpr (PREC == P_FP32C) x += (double)s.xl[c];
        return x;
    };
    auto vel = [&](const St<PREC> &s, int c) {
        double v = (double)s.v[c];
        if constexpr (PREC == P_FP32C) v += (double)s.vl[c];
        return v;
    };
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.n; g += stride) {
        const St<PREC> s = load_state<PREC>(a.state, g);
        double m = (double)ms[g];
        double x[3] = {pos(s, 0), pos(s, 1), pos(s, 2)};
        double v[3] = {vel(s, 0), vel(s, 1), vel(s, 2)};
        double vn = nrm3(v[0], v[1], v[2]);
        q[1] += (0.5 * m) * (vn * vn);
        q[2] += (a.g_mag * x[2]) * m;
        double p[3] = {v[0] * m, v[1] * m, v[2] * m};
        q[3] += p[0];
        q[4] += p[1];
        q[5] += p[2];
        q[6] += p[1] * x[2] - p[2] * x[1];
        q[7] += x[0] * p[2] - p[0] * x[2];
        q[8] += p[0] * x[1] - p[1] * x[0];
    }
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < a.ns; s += stride) {
        int32_t l = a.sl[s], r = a.sr[s];
        if (l < 0) continue;
        const St<PREC> sl = load_state<PREC>(a.state, l), sr = load_state<PREC>(a.state, r);
        double d0 = pos(sl, 0) - pos(sr, 0), d1 = pos(sl, 1) - pos(sr, 1), d2 = pos(sl, 2) - pos(sr, 2);
        double x = nrm3(d0, d1, d2) - a.srest[s];
        q[0] += (a.sk[s] * (x * x)) / 2;
    }
#pragma unroll
    for (int k = 0; k < kDiagQ; k++) red[k][threadIdx.x] = q[k];
    __syncthreads();
    for (int w = 128; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < kDiagQ; k++) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kDiagQ) a.partials[blockIdx.x * kDiagQ + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void __launch_bounds__(256) k_diag2(DiagArgs a) {
    __shared__ double red[kDiagQ][256];
    for (int k = 0; k < kDiagQ; k++) {
        double s = 0.0;
        for (int b = threadIdx.x; b < kDiagBlocks; b += 256) s += a.partials[b * kDiagQ + k];
        red[k][threadIdx.x] = s;
    }
    __syncthreads();
    for (int w = 128; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < kDiagQ; k++) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kDiagQ) a.out[threadIdx.x] = red[threadIdx.x][0];
}

}  // namespace


cudaError_t launch_export_f32(int precision, const XferArgs &a, float *out, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((a.count + 255) / 256);
    switch (precision) {
        case P_FP64: k_export_f32<P_FP64><<<blocks, 256, 0, s>>>(a, out); break;
        case P_FP32: k_export_f32<P_FP32><<<blocks, 256, 0, s>>>(a, out); break;
        default: k_export_f32<P_FP32C><<<blocks, 256, 0, s>>>(a, out); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_gather(int precision, const XferArgs &a, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    int blocks = (int)((a.count + 255) / 256);
    switch (precision) {
        case P_FP64: k_gather<P_FP64><<<blocks, 256, 0, s>>>(a); break;
        case P_FP32: k_gather<P_FP32><<<blocks, 256, 0, s>>>(a); break;
        default: k_gather<P_FP32C><<<blocks, 256, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_scatter(int precision, const XferArgs &a, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    int blocks = (int)((a.count + 255) / 256);
    switch (precision) {
        case P_FP64: k_scatter<P_FP64><<<blocks, 256, 0, s>>>(a); break;
        case P_FP32: k_scatter<P_FP32><<<blocks, 256, 0, s>>>(a); break;
        default: k_scatter<P_FP32C><<<blocks, 256, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_diag(int precision, const DiagArgs &a, cudaStream_t s) {
    switch (precision) {
        case P_FP64: k_diag1<P_FP64><<<kDiagBlocks, 256, 0, s>>>(a); break;
        case P_FP32: k_diag1<P_FP32><<<kDiagBlocks, 256, 0, s>>>(a); break;
        default: k_diag1<P_FP32C><<<kDiagBlocks, 256, 0, s>>>(a); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_diag2<<<1, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace tg
