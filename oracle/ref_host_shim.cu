// ref_host_shim.cu -- C entry points onto the reference's own host-callable
// code, compiled from the reference sources by oracle/build_ref.sh into
// oracle/_ref/libtitan_ref_host.so.  TEST INFRASTRUCTURE ONLY: used to pin the
// oracle (tests/golden/make_golden.py); nothing in the product links it.
#include <cstdint>
#include <map>

#include "object.h"
#include "mass.h"
#include "spring.h"
#include "vec.h"

using titan::Vec;

extern "C" {

int64_t ref_lattice_springs(int nx, int ny, int nz) {
    titan::Lattice L(Vec(0, 0, 0), Vec(1, 1, 1), nx, ny, nz);
    int64_t ns = (int64_t)L.springs.size();
    for (auto *s : L.springs) delete s;
    for (auto *m : L.masses) delete m;
    return ns;
}

// titan::Lattice (src/object.cu:232-293) flattened into arrays.
int ref_lattice(const double *c, const double *d, int nx, int ny, int nz, double *pos, int32_t *left,
                int32_t *right, double *rest) {
    titan::Lattice L(Vec(c[0], c[1], c[2]), Vec(d[0], d[1], d[2]), nx, ny, nz);
    std::map<const titan::Mass *, int32_t> id;
    for (size_t i = 0; i < L.masses.size(); i++) {
        id[L.masses[i]] = (int32_t)i;
        for (int k = 0; k < 3; k++) pos[3 * i + k] = L.masses[i]->pos[k];
    }
    for (size_t j = 0; j < L.springs.size(); j++) {
        left[j] = id[L.springs[j]->_left];
        right[j] = id[L.springs[j]->_right];
        rest[j] = L.springs[j]->_rest;
    }
    for (auto *s : L.springs) delete s;
    for (auto *m : L.masses) delete m;
    return 0;
}

static void load(titan::CUDA_MASS &m, const double *pos, const double *vel, const double *force) {
    m.pos = Vec(pos[0], pos[1], pos[2]);
    m.vel = Vec(vel[0], vel[1], vel[2]);
    m.force = Vec(force[0], force[1], force[2]);
}
static void store(const titan::CUDA_MASS &m, double *vel, double *force) {
    for (int k = 0; k < 3; k++) {
        force[k] = m.force[k];
        if (vel) vel[k] = m.vel[k];
    }
}

// createPlane(n, off, fk, fs) -> ContactPlane -> CudaContactPlane::applyForce
void ref_plane_apply(const double *n, double off, double fk, double fs, const double *pos,
                     const double *vel, double *force) {
    titan::ContactPlane p(Vec(n[0], n[1], n[2]), off);
    p._FRICTION_K = fk;
    p._FRICTION_S = fs;
    titan::CudaContactPlane cp(p);
    titan::CUDA_MASS m;
    load(m, pos, vel, force);
    cp.applyForce(&m);
    store(m, nullptr, force);
}

void ref_ball_apply(const double *c, double r, const double *pos, double *force) {
    titan::CudaBall b(Vec(c[0], c[1], c[2]), r);
    titan::CUDA_MASS m;
    double zero[3] = {0, 0, 0};
    load(m, pos, zero, force);
    b.applyForce(&m);
    store(m, nullptr, force);
}

void ref_constraint_plane_apply(const double *n, double fr, const double *pos, double *vel, double *force) {
    titan::CudaConstraintPlane p(Vec(n[0], n[1], n[2]), fr);
    titan::CUDA_MASS m;
    load(m, pos, vel, force);
    p.applyForce(&m);
    store(m, vel, force);
}

void ref_direction_apply(const double *t, double fr, const double *pos, double *vel, double *force) {
    titan::CudaDirection p(Vec(t[0], t[1], t[2]), fr);
    titan::CUDA_MASS m;
    load(m, pos, vel, force);
    p.applyForce(&m);
    store(m, vel, force);
}

// ContactPlane's constructor normalisation (include/Titan/object.h:103).
void ref_normalize(const double *v, double *out) {
    titan::ContactPlane p(Vec(v[0], v[1], v[2]), 0.0);
    for (int k = 0; k < 3; k++) out[k] = p._normal[k];
}

}  // extern "C"
