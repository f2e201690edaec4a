// ref_gpu_shim.cu -- device-side glue for running the reference's own CUDA
// kernels (src/sim.cu:1046-1080 computeSpringForces, src/sim.cu:1093-1169
// massForcesAndUpdate) outside titan::Simulation.  TEST INFRASTRUCTURE
// ONLY: oracle/build_ref.sh compiles it with the reference sources into one
// device-linked cubin, oracle/_ref/titan_ref_kernels.cubin; the host side
// (oracle/ref_gpu_harness.cpp) loads that cubin with the driver API.
//
// The reference builds its device records one object at a time (createMass /
// createSpring, src/sim.cu:223-341, then CUDA_MASS(Mass&) and
// CUDA_SPRING(const Spring&, ...), src/mass.cu, src/spring.cu).  These
// kernels fill the same records from structure-of-arrays inputs, with the
// values those constructors give (T = 0, acc = force = extern force = 0
// unless given, valid = true, no local constraints, drag 0), so that a
// 10^6-mass scene is set up in milliseconds instead of 10^7 cudaMalloc calls.
#include <cstdint>

#include "mass.h"
#include "object.h"
#include "spring.h"
#include "vec.h"

using titan::CUDA_MASS;
using titan::CUDA_SPRING;
using titan::CudaBall;
using titan::CudaContactPlane;
using titan::Vec;

extern "C" {

// Layout facts the host harness needs: sizes of the records and of the two
// by-value kernel arguments (Vec, CUDA_GLOBAL_CONSTRAINTS).
__global__ void ref_gpu_sizes(int64_t *out) {
    out[0] = sizeof(CUDA_MASS);
    out[1] = sizeof(CUDA_SPRING);
    out[2] = sizeof(CudaContactPlane);
    out[3] = sizeof(CudaBall);
    out[4] = sizeof(Vec);
    out[5] = sizeof(titan::CUDA_GLOBAL_CONSTRAINTS);
    titan::CUDA_GLOBAL_CONSTRAINTS c;
    out[6] = (int64_t)((char *)&c.d_balls - (char *)&c);
    out[7] = (int64_t)((char *)&c.num_planes - (char *)&c);
    out[8] = (int64_t)((char *)&c.num_balls - (char *)&c);
}

// Mass records and the pointer array the kernels take (createMassPointers,
// src/sim.cu:821-830, does the pointer part).  pos, vel, ext are
// xyz-interleaved; vel, ext, fixed, drag may be null.
__global__ void ref_gpu_fill_masses(CUDA_MASS *data, CUDA_MASS **ptrs, int n, const double *pos,
                                    const double *vel, const double *m, const double *ext,
                                    const uint8_t *fixed, const double *drag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    CUDA_MASS &r = data[i];
    r.m = m[i];
    r.T = 0.0;
    r.pos = Vec(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    r.vel = vel ? Vec(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]) : Vec(0, 0, 0);
    r.acc = Vec(0, 0, 0);
    r.force = Vec(0, 0, 0);
    r.extern_force = ext ? Vec(ext[3 * i], ext[3 * i + 1], ext[3 * i + 2]) : Vec(0, 0, 0);
    r.valid = true;
    r.constraints.contact_plane = nullptr;
    r.constraints.constraint_plane = nullptr;
    r.constraints.ball = nullptr;
    r.constraints.direction = nullptr;
    r.constraints.drag_coefficient = drag ? (int)drag[i] : 0;
    r.constraints.fixed = fixed ? fixed[i] != 0 : false;
    r.constraints.num_contact_planes = 0;
    r.constraints.num_balls = 0;
    r.constraints.num_constraint_planes = 0;
    r.constraints.num_directions = 0;
    ptrs[i] = &r;
}

// Spring records (left/right index -1: no mass attached) and their pointer
// array (createSpringPointers, src/sim.cu:871-880).
__global__ void ref_gpu_fill_springs(CUDA_SPRING *data, CUDA_SPRING **ptrs, int ns, CUDA_MASS *masses,
                                     const int32_t *left, const int32_t *right, const double *k,
                                     const double *rest, const double *damping, const int32_t *type,
                                     const double *omega) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ns) return;
    CUDA_SPRING &s = data[j];
    s._left = left[j] >= 0 ? masses + left[j] : nullptr;
    s._right = right[j] >= 0 ? masses + right[j] : nullptr;
    s._k = k[j];
    s._rest = rest[j];
    s._type = type ? (titan::SpringType)type[j] : titan::PASSIVE_SOFT;
    s._omega = omega ? omega[j] : 0.0;
    s._damping = damping ? damping[j] : 0.0;
    ptrs[j] = &s;
}

// Global constraints as createPlane / createBall leave them on the device
// (src/sim.cu:1998-2035): 6 doubles per plane (normal, offset, friction_k,
// friction_s; the normal is normalised by the reference's constructor) and
// 4 per ball (centre, radius).
__global__ void ref_gpu_fill_constraints(CudaContactPlane *planes, int np, const double *pp, CudaBall *balls,
                                         int nb, const double *bp) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int j = 0; j < np; j++) {
        const double *q = pp + 6 * j;
        // this constructor normalises the normal once, as ContactPlane's does
        planes[j] = CudaContactPlane(Vec(q[0], q[1], q[2]), q[3]);
        planes[j]._FRICTION_K = q[4];
        planes[j]._FRICTION_S = q[5];
    }
    for (int j = 0; j < nb; j++) {
        const double *q = bp + 4 * j;
        balls[j] = CudaBall(Vec(q[0], q[1], q[2]), q[3]);
    }
}

// Positions, velocities, accelerations and local times back to arrays.
__global__ void ref_gpu_read_masses(const CUDA_MASS *data, int n, double *pos, double *vel, double *acc,
                                    double *T) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const CUDA_MASS &r = data[i];
    for (int c = 0; c < 3; c++) {
        pos[3 * i + c] = r.pos[c];
        vel[3 * i + c] = r.vel[c];
        acc[3 * i + c] = r.acc[c];
    }
    T[i] = r.T;
}

}  // extern "C"
