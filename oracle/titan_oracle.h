/*
 * titan_oracle.h -- CPU FP64 restatement of Titan's mass-spring time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA path is checked
 * against; it is never linked into, loaded by, or called from the product
 * library (titan_gb300/).  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py may use it.
 *
 * Every function restates one piece of the reference (jacobaustin123/Titan);
 * the file:line it follows is given beside each declaration.
 */
#ifndef TITAN_ORACLE_H
#define TITAN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Spring actuation types, same numbering as include/Titan/spring.h:17. */
enum { TO_PASSIVE_SOFT = 0, TO_PASSIVE_STIFF = 1,
       TO_ACTIVE_CONTRACT_THEN_EXPAND = 2, TO_ACTIVE_EXPAND_THEN_CONTRACT = 3 };

/* Local constraint types, same numbering as include/Titan/object.h:223-225. */
enum { TO_CONSTRAINT_PLANE = 0, TO_CONTACT_PLANE = 1, TO_BALL = 2, TO_DIRECTION = 3 };

/* Accumulation orders for the per-mass spring-force sum.  The reference
 * accumulates with FP64 atomics (src/vec.cu:33-37), so any serialisation of
 * the springs is a legal reference result. */
enum {
    TO_ORDER_ASCENDING = 0,   /* springs in index order == per-mass CSR order */
    TO_ORDER_DESCENDING = 1,  /* another legal atomic serialisation          */
    TO_ORDER_ATOMIC_OMP = 2,  /* OpenMP parallel with atomics (timing only)  */
    TO_ORDER_DEVICE = 3       /* ascending, but masses with degree > heavy_threshold
                                 use the lane-strided + xor-tree order of the
                                 CUDA kernel's warp-cooperative path         */
};

typedef struct {
    /* masses (xyz interleaved, 3*n_masses doubles) */
    int64_t n_masses;
    double *pos, *vel, *acc, *force;
    const double *ext;        /* external force, may be NULL (= zero)            */
    const double *m;
    double *T;                /* per-mass local time, may be NULL                */
    const uint8_t *fixed;     /* may be NULL                                     */
    const int32_t *drag;      /* truncated drag coefficient, may be NULL         */
    /* local constraints: records of mass i are lc_ptr[i]..lc_ptr[i+1], already
       in application order (contact planes, balls, constraint planes, directions);
       vectors already normalised as the reference constructors do.  May be NULL. */
    const int64_t *lc_ptr;
    const int32_t *lc_type;
    const double *lc_vec;     /* 3 per record */
    const double *lc_num;
    /* springs */
    int64_t n_springs;
    const int32_t *left, *right;   /* -1 = no mass attached                     */
    const double *k, *rest, *damping;
    const int32_t *type;           /* may be NULL (all passive)                 */
    const double *omega;           /* may be NULL                               */
    const double *amp;             /* may be NULL (reference amplitude 0.2)     */
    const double *phase;           /* may be NULL (reference phase 0)           */
    /* global constraints; plane normals already normalised */
    int32_t n_planes;
    const double *plane_n, *plane_off, *plane_fk, *plane_fs;
    int32_t n_balls;
    const double *ball_c, *ball_r;
    /* per-body ground planes (an extension: a friction contact plane acting on
       the masses of one body only), applied after the global balls.  mass_bp[i]
       is the plane of mass i or -1; may be NULL. */
    const int32_t *mass_bp;
    const double *bp_n, *bp_off, *bp_fk, *bp_fs;
    /* globals */
    double g[3];
    double dt;
    double T_global;               /* host-accumulated simulation time           */
    int32_t heavy_threshold;       /* for TO_ORDER_DEVICE                        */
    int32_t integrator;            /* TO_EULER (default), TO_VERLET, TO_RK2      */
} to_scene;

/* Integrators of massForcesAndUpdate (src/sim.cu:1141-1166): the default
 * symplectic Euler, and the compile-time VERLET and RK2 variants.  VERLET
 * keeps the acceleration as state (acc must not be NULL); RK2 evaluates the
 * spring forces twice per step, at T and at T + dt/2 (src/sim.cu:1572-1583). */
enum { TO_EULER = 0, TO_VERLET = 1, TO_RK2 = 2 };

/* One time step == computeSpringForces (src/sim.cu:1046-1080) followed by
 * massForcesAndUpdate (src/sim.cu:1093-1169, CONSTRAINTS on) and the host
 * time update T += dt (src/sim.cu:1590); with RK2 both twice, T += dt/2
 * after each (src/sim.cu:1572-1583).  Returns 0 on success. */
int to_step(to_scene *s, int64_t nsteps, int order, int nthreads);

/* Point-in-mesh classification of STL import (stl::stlFile::inside,
 * include/Titan/stlparser.h:213-276): inside when more than half of num_rays
 * rays cross the mesh an odd number of times; ray r of point i is three
 * uniform values in [-1000, 1000) from SplitMix64(seed, i, r) divided by its
 * norm (the reference draws them with rand()).  tri: 9 doubles per triangle;
 * pts: 3 per point; inside: 1 byte per point.  num_rays <= 64. */
int to_stl_inside(const double *tri, int64_t ntri, const double *pts, int64_t npts, int num_rays, uint64_t seed,
                  uint8_t *inside, int nthreads);

/* Spring force on the RIGHT endpoint (src/sim.cu:1054-1065); the left one gets
 * its negation. */
void to_spring_force(const double *pl, const double *pr, const double *vl, const double *vr,
                     double k, double rest, double damping, int32_t type, double omega,
                     double amp, double phase, double t, double out[3]);

/* Constraint force functions, restating src/object.cu:53-56 (ball),
 * :73-106 (contact plane), :115-124 (constraint plane), :133-141 (direction).
 * They update force (and, for the last two, vel) in place. */
void to_ball_apply(const double c[3], double r, const double pos[3], double force[3]);
void to_plane_apply(const double n[3], double off, double fk, double fs,
                    const double pos[3], const double vel[3], double force[3]);
void to_constraint_plane_apply(const double n[3], double friction,
                               double vel[3], double force[3]);
void to_direction_apply(const double t[3], double friction, double vel[3], double force[3]);

/* v / |v| exactly as the reference constructors normalise (object.h:103). */
void to_normalize(const double v[3], double out[3]);

/* Lattice builder, restating src/object.cu:232-293.  pos must hold 3*nx*ny*nz
 * doubles; left/right/rest hold to_lattice_springs(nx,ny,nz) entries. */
int64_t to_lattice_springs(int nx, int ny, int nz);
void to_lattice(const double center[3], const double dims[3], int nx, int ny, int nz,
                double *pos, int32_t *left, int32_t *right, double *rest);

/* Energy as test/testutil/utils.h:12-30 (gravity magnitude passed in) and
 * momentum as :32-43 (linear and angular kept apart). out: [spring PE,
 * kinetic, gravity PE, total]. */
void to_energy(const to_scene *s, double g_mag, double out[4]);
void to_momentum(const to_scene *s, double lin[3], double ang[3]);

#ifdef __cplusplus
}
#endif
#endif
