// ref_gpu_harness.cpp -- runs the reference's own CUDA kernels on a GPU.
//
// TEST INFRASTRUCTURE ONLY (parity tests and the reference-kernel timing in
// bench.py); nothing in the product links it.  It loads the cubin that
// oracle/build_ref.sh device-links from the reference sources (src/sim.cu,
// src/object.cu, src/mass.cu, src/spring.cu, src/vec.cu) plus
// oracle/ref_gpu_shim.cu, fills the reference's device records with the
// shim's kernels, and steps the scene exactly as Simulation::execute()
// does (src/sim.cu:1568-1583, Euler build): per step
//     computeSpringForces<<<ceil(Ns / 1024), 1024>>>(d_spring, Ns, T);
//     massForcesAndUpdate<<<ceil(Nm / 1024), 1024>>>(d_mass, Nm, dt, T, g, c);
//     T += dt;                                     (host double)
// with THREADS_PER_BLOCK = 1024 and grids capped at MAX_BLOCKS = 65535
// (include/Titan/sim.h:31-32, src/sim.cu:1464-1475), optionally preceded
// by the cudaDeviceSynchronize() execute() issues before every step
// (src/sim.cu:1570).  Only the CUDA driver API is used, so this file needs
// none of the reference's headers and builds wherever the CUDA toolkit is.
#include <cuda.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int kThreads = 1024;     // THREADS_PER_BLOCK
constexpr int kMaxBlocks = 65535;  // MAX_BLOCKS

const char *kSpringKernel = "_ZN5titan19computeSpringForcesEPPNS_11CUDA_SPRINGEid";
const char *kMassKernel = "_ZN5titan19massForcesAndUpdateEPPNS_9CUDA_MASSEiddNS_3VecENS_23CUDA_GLOBAL_CONSTRAINTSE";

struct Harness {
    CUcontext ctx = nullptr;
    CUdevice dev = 0;
    CUmodule mod = nullptr;
    CUfunction f_spring = nullptr, f_mass = nullptr, f_sizes = nullptr, f_fill_m = nullptr, f_fill_s = nullptr,
               f_fill_c = nullptr, f_read = nullptr;
    int64_t sizes[9] = {};
    std::vector<CUdeviceptr> allocs;
    CUdeviceptr masses = 0, mass_ptrs = 0, springs = 0, spring_ptrs = 0, planes = 0, balls = 0;
    int n = 0, ns = 0, np = 0, nb = 0;
    double dt = 1e-4, T = 0.0, g[3] = {0, 0, -9.81};
    std::string err;
};

Harness H;

bool ck(CUresult r, const char *what) {
    if (r == CUDA_SUCCESS) return true;
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    H.err = std::string(what) + ": " + (s ? s : "unknown CUDA error");
    return false;
}

CUdeviceptr dalloc(size_t bytes) {
    CUdeviceptr p = 0;
    if (!ck(cuMemAlloc(&p, bytes ? bytes : 16), "cuMemAlloc")) return 0;
    H.allocs.push_back(p);
    return p;
}

template <typename T>
CUdeviceptr upload(const T *host, size_t count) {
    if (!host) return 0;
    CUdeviceptr p = dalloc(count * sizeof(T));
    if (p && !ck(cuMemcpyHtoD(p, host, count * sizeof(T)), "upload")) return 0;
    return p;
}

void release() {
    for (CUdeviceptr p : H.allocs) cuMemFree(p);
    H.allocs.clear();
    H.masses = H.mass_ptrs = H.springs = H.spring_ptrs = H.planes = H.balls = 0;
}

int grid(int count) {
    int b = (count + kThreads - 1) / kThreads;
    if (b > kMaxBlocks) b = kMaxBlocks;
    if (b < 1) b = 1;
    return b;
}

bool launch(CUfunction f, int blocks, int threads, void **args) {
    return ck(cuLaunchKernel(f, blocks, 1, 1, threads, 1, 1, 0, nullptr, args, nullptr), "cuLaunchKernel");
}

// One execute() iteration (Euler build).
bool one_step() {
    int ns = H.ns, n = H.n;
    double T = H.T, dt = H.dt;
    void *a1[] = {&H.spring_ptrs, &ns, &T};
    if (!launch(H.f_spring, grid(ns), kThreads, a1)) return false;
    // Vec (3 doubles) and CUDA_GLOBAL_CONSTRAINTS by value, laid out as the
    // shim's ref_gpu_sizes reported
    alignas(8) unsigned char vec[24];
    std::memcpy(vec, H.g, 24);
    alignas(8) unsigned char cons[64] = {};
    std::memcpy(cons, &H.planes, 8);
    std::memcpy(cons + H.sizes[6], &H.balls, 8);
    std::memcpy(cons + H.sizes[7], &H.np, 4);
    std::memcpy(cons + H.sizes[8], &H.nb, 4);
    void *a2[] = {&H.mass_ptrs, &n, &dt, &T, vec, cons};
    if (!launch(H.f_mass, grid(n), kThreads, a2)) return false;
    H.T = H.T + H.dt;
    return true;
}

}  // namespace

extern "C" {

const char *refgpu_error(void) { return H.err.c_str(); }

// Loads the cubin into the primary context of CUDA device `device` (the
// context the CUDA runtime uses).  Returns 0 on success.
int refgpu_open(const char *cubin_path, int device) {
    if (!ck(cuInit(0), "cuInit")) return 1;
    if (!ck(cuDeviceGet(&H.dev, device), "cuDeviceGet")) return 1;
    if (!ck(cuDevicePrimaryCtxRetain(&H.ctx, H.dev), "cuDevicePrimaryCtxRetain")) return 1;
    if (!ck(cuCtxSetCurrent(H.ctx), "cuCtxSetCurrent")) return 1;
    if (H.mod) return 0;
    if (!ck(cuModuleLoad(&H.mod, cubin_path), "cuModuleLoad")) return 1;
    struct {
        CUfunction *f;
        const char *name;
    } fs[] = {{&H.f_spring, kSpringKernel}, {&H.f_mass, kMassKernel}, {&H.f_sizes, "ref_gpu_sizes"},
              {&H.f_fill_m, "ref_gpu_fill_masses"}, {&H.f_fill_s, "ref_gpu_fill_springs"},
              {&H.f_fill_c, "ref_gpu_fill_constraints"}, {&H.f_read, "ref_gpu_read_masses"}};
    for (auto &x : fs)
        if (!ck(cuModuleGetFunction(x.f, H.mod, x.name), x.name)) return 1;
    CUdeviceptr d = dalloc(9 * sizeof(int64_t));
    if (!d) return 1;
    void *a[] = {&d};
    if (!launch(H.f_sizes, 1, 1, a)) return 1;
    if (!ck(cuMemcpyDtoH(H.sizes, d, sizeof(H.sizes)), "sizes")) return 1;
    release();
    if (H.sizes[4] != 24 || H.sizes[5] > 64 || H.sizes[6] + 8 > H.sizes[5] || H.sizes[8] + 4 > H.sizes[5]) {
        H.err = "unexpected reference record layout";
        return 1;
    }
    return 0;
}

// sizes of CUDA_MASS, CUDA_SPRING, CudaContactPlane, CudaBall, Vec,
// CUDA_GLOBAL_CONSTRAINTS (bytes)
void refgpu_sizes(int64_t out[6]) { std::memcpy(out, H.sizes, 6 * sizeof(int64_t)); }

// Uploads a scene (creation order; pos, vel, ext xyz-interleaved; 6 doubles
// per plane: normal, offset, friction_k, friction_s; 4 per ball: centre,
// radius).  vel, ext, fixed, drag, damping, type, omega may be null.
int refgpu_setup(int64_t n, const double *pos, const double *vel, const double *m, const double *ext,
                 const uint8_t *fixed, const double *drag, int64_t ns, const int32_t *left, const int32_t *right,
                 const double *k, const double *rest, const double *damping, const int32_t *type,
                 const double *omega, int np, const double *planes, int nb, const double *balls, const double *g,
                 double dt) {
    if (!H.mod) {
        H.err = "refgpu_open first";
        return 1;
    }
    // the fill kernels cover kMaxBlocks * kThreads records, as the
    // reference's own launches do
    const int64_t lim = (int64_t)kMaxBlocks * kThreads;
    if (n <= 0 || n > lim || ns < 0 || ns > lim || np < 0 || nb < 0) {
        H.err = "scene size out of range";
        return 1;
    }
    for (int64_t j = 0; j < ns; j++)
        if (left[j] < -1 || left[j] >= n || right[j] < -1 || right[j] >= n) {
            H.err = "spring end out of range";
            return 1;
        }
    if (!ck(cuCtxSetCurrent(H.ctx), "cuCtxSetCurrent")) return 1;
    release();
    H.n = (int)n;
    H.ns = (int)ns;
    H.np = np;
    H.nb = nb;
    H.dt = dt;
    H.T = 0.0;
    std::memcpy(H.g, g, sizeof(H.g));
    H.masses = dalloc((size_t)n * H.sizes[0]);
    H.mass_ptrs = dalloc((size_t)n * 8);
    H.springs = dalloc((size_t)(ns > 0 ? ns : 1) * H.sizes[1]);
    H.spring_ptrs = dalloc((size_t)(ns > 0 ? ns : 1) * 8);
    H.planes = dalloc((size_t)(np > 0 ? np : 1) * H.sizes[2]);
    H.balls = dalloc((size_t)(nb > 0 ? nb : 1) * H.sizes[3]);
    if (!H.masses || !H.mass_ptrs || !H.springs || !H.spring_ptrs || !H.planes || !H.balls) return 1;
    CUdeviceptr dpos = upload(pos, 3 * n), dvel = upload(vel, 3 * n), dm = upload(m, n), dext = upload(ext, 3 * n);
    CUdeviceptr dfix = upload(fixed, n), ddrag = upload(drag, n);
    CUdeviceptr dl = upload(left, ns), dr = upload(right, ns), dk = upload(k, ns), drest = upload(rest, ns);
    CUdeviceptr ddamp = upload(damping, ns), dtype = upload(type, ns), domega = upload(omega, ns);
    CUdeviceptr dpp = upload(planes, 6 * (size_t)np), dbp = upload(balls, 4 * (size_t)nb);
    if (!dpos || !dm || (ns > 0 && (!dl || !dr || !dk || !drest))) return 1;
    int ni = (int)n, nsi = (int)ns;
    void *am[] = {&H.masses, &H.mass_ptrs, &ni, &dpos, &dvel, &dm, &dext, &dfix, &ddrag};
    if (!launch(H.f_fill_m, grid(ni), kThreads, am)) return 1;
    if (ns > 0) {
        void *as[] = {&H.springs, &H.spring_ptrs, &nsi, &H.masses, &dl, &dr, &dk, &drest, &ddamp, &dtype, &domega};
        if (!launch(H.f_fill_s, grid(nsi), kThreads, as)) return 1;
    }
    void *ac[] = {&H.planes, &np, &dpp, &H.balls, &nb, &dbp};
    if (!launch(H.f_fill_c, 1, 1, ac)) return 1;
    if (!ck(cuCtxSynchronize(), "setup")) return 1;
    return 0;
}

// nsteps iterations; sync_each: cudaDeviceSynchronize before every step as
// execute() does.  Asynchronous when sync_each is 0.
int refgpu_step(int64_t nsteps, int sync_each) {
    if (!ck(cuCtxSetCurrent(H.ctx), "cuCtxSetCurrent")) return 1;
    for (int64_t i = 0; i < nsteps; i++) {
        if (sync_each && !ck(cuCtxSynchronize(), "step sync")) return 1;
        if (!one_step()) return 1;
    }
    return 0;
}

// Milliseconds of nsteps iterations measured with CUDA events on the
// default stream (-1 on error).
double refgpu_time_steps(int64_t nsteps, int sync_each) {
    CUevent e0, e1;
    if (!ck(cuEventCreate(&e0, CU_EVENT_DEFAULT), "event") || !ck(cuEventCreate(&e1, CU_EVENT_DEFAULT), "event"))
        return -1;
    if (!ck(cuCtxSynchronize(), "sync")) return -1;
    cuEventRecord(e0, nullptr);
    if (refgpu_step(nsteps, sync_each)) return -1;
    cuEventRecord(e1, nullptr);
    if (!ck(cuEventSynchronize(e1), "event sync")) return -1;
    float ms = 0;
    cuEventElapsedTime(&ms, e0, e1);
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    return ms;
}

double refgpu_time(void) { return H.T; }

// Positions, velocities, accelerations (xyz-interleaved) and local times.
int refgpu_read(double *pos, double *vel, double *acc, double *T) {
    if (!ck(cuCtxSetCurrent(H.ctx), "cuCtxSetCurrent")) return 1;
    const size_t n = (size_t)H.n;
    CUdeviceptr d = 0;
    if (!ck(cuMemAlloc(&d, 10 * n * sizeof(double)), "cuMemAlloc")) return 1;
    CUdeviceptr dp = d, dv = d + 3 * n * 8, da = d + 6 * n * 8, dT = d + 9 * n * 8;
    int ni = H.n;
    void *a[] = {&H.masses, &ni, &dp, &dv, &da, &dT};
    bool ok = launch(H.f_read, grid(ni), kThreads, a) && ck(cuCtxSynchronize(), "read");
    std::vector<double> h(10 * n);
    ok = ok && ck(cuMemcpyDtoH(h.data(), d, h.size() * sizeof(double)), "read");
    cuMemFree(d);
    if (!ok) return 1;
    if (pos) std::memcpy(pos, h.data(), 3 * n * 8);
    if (vel) std::memcpy(vel, h.data() + 3 * n, 3 * n * 8);
    if (acc) std::memcpy(acc, h.data() + 6 * n, 3 * n * 8);
    if (T) std::memcpy(T, h.data() + 9 * n, n * 8);
    return 0;
}

void refgpu_close(void) {
    if (H.ctx) cuCtxSetCurrent(H.ctx);
    release();
    if (H.mod) cuModuleUnload(H.mod);
    H.mod = nullptr;
    if (H.ctx) cuDevicePrimaryCtxRelease(H.dev);
    H.ctx = nullptr;
}

}  // extern "C"
