/*
 * titan_oracle.c -- CPU FP64 restatement of Titan's mass-spring time step.
 *
 * TEST INFRASTRUCTURE ONLY (see titan_oracle.h).  Compiled with
 * -ffp-contract=off so that every product and sum is rounded exactly once,
 * in the order written, on both x86_64 and aarch64 hosts.
 *
 * Parity pins: the lattice builder and the constraint force functions are
 * checked bit-for-bit against the reference's own host-callable code
 * (src/object.cu compiled from the reference sources by oracle/build_ref.sh,
 * fixtures in tests/golden/); the step is checked against the known answers
 * of tests/test_oracle.py and against the reference's test tolerances
 * (test/physics/ in the reference).
 */
#include "titan_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Reference: __device__ const double NORMAL = 20000 (src/object.cu:26). */
#define TO_NORMAL 20000.0

/* |v| = sqrt(pow(x,2)+pow(y,2)+pow(z,2)) (include/Titan/vec.h:149); pow(x, 2)
 * of a double is the exactly rounded square, i.e. x*x. */
static double nrm3(const double v[3]) {
    double a = v[0] * v[0];
    double b = v[1] * v[1];
    double c = v[2] * v[2];
    return sqrt((a + b) + c);
}

/* dot(a, b) = (a*b).sum() (src/vec.cu:39-41, vec.h:153). */
static double dot3(const double a[3], const double b[3]) {
    double x = a[0] * b[0];
    double y = a[1] * b[1];
    double z = a[2] * b[2];
    return (x + y) + z;
}

void to_normalize(const double v[3], double out[3]) {
    double n = nrm3(v);
    out[0] = v[0] / n;
    out[1] = v[1] / n;
    out[2] = v[2] / n;
}

/* src/sim.cu:1054-1065.  temp = right.pos - left.pos; scale from actuation;
 * F = k (rest*scale - |temp|) temp/|temp| + ((v_l - v_r).(temp/|temp|)) c temp/|temp|.
 * The amplitude and phase are extensions: amp = 0.2, phase = 0 reproduce the
 * reference's 1 -/+ 0.2 sin(omega t) exactly. */
void to_spring_force(const double *pl, const double *pr, const double *vl, const double *vr,
                     double k, double rest, double damping, int32_t type, double omega,
                     double amp, double phase, double t, double out[3]) {
    double d[3] = {pr[0] - pl[0], pr[1] - pl[1], pr[2] - pl[2]};
    double scale = 1.0;
    if (type == TO_ACTIVE_CONTRACT_THEN_EXPAND) {
        double th = omega * t;
        th = th + phase;
        double a = amp * sin(th);
        scale = 1.0 - a;
    } else if (type == TO_ACTIVE_EXPAND_THEN_CONTRACT) {
        double th = omega * t;
        th = th + phase;
        double a = amp * sin(th);
        scale = 1.0 + a;
    }
    double n = nrm3(d);
    double u[3] = {d[0] / n, d[1] / n, d[2] / n};
    double rs = rest * scale;
    double fs = k * (rs - n);
    out[0] = u[0] * fs;
    out[1] = u[1] * fs;
    out[2] = u[2] * fs;
    double dv[3] = {vl[0] - vr[0], vl[1] - vr[1], vl[2] - vr[2]};
    double dd = dot3(dv, u) * damping;
    out[0] = out[0] + u[0] * dd;
    out[1] = out[1] + u[1] * dd;
    out[2] = out[2] + u[2] * dd;
}

/* src/object.cu:53-56: constant-magnitude push when inside the ball. */
void to_ball_apply(const double c[3], double r, const double pos[3], double force[3]) {
    double d[3] = {pos[0] - c[0], pos[1] - c[1], pos[2] - c[2]};
    double dist = nrm3(d);
    if (dist <= r) {
        force[0] = force[0] + (TO_NORMAL * d[0]) / dist;
        force[1] = force[1] + (TO_NORMAL * d[1]) / dist;
        force[2] = force[2] + (TO_NORMAL * d[2]) / dist;
    } else {
        force[0] = force[0] + 0.0;
        force[1] = force[1] + 0.0;
        force[2] = force[2] + 0.0;
    }
}

/* src/object.cu:73-106: penalty contact plus kinetic / static friction.  The
 * friction uses the force accumulated so far (springs, gravity, external and
 * earlier constraints), as the reference does. */
void to_plane_apply(const double n[3], double off, double fk, double fs,
                    const double pos[3], const double vel[3], double force[3]) {
    double disp = dot3(pos, n) - off;
    double fdn = dot3(force, n);
    double fn[3] = {n[0] * fdn, n[1] * fdn, n[2] * fdn};
    if (disp < 0 && (fs > 0 || fk > 0)) {
        double vdn = dot3(vel, n);
        double vp[3] = {vel[0] - n[0] * vdn, vel[1] - n[1] * vdn, vel[2] - n[2] * vdn};
        double vnorm = nrm3(vp);
        if (vnorm > 1e-16) {
            double fmag = fk * nrm3(fn);
            force[0] = force[0] - (vp[0] * fmag) / vnorm;
            force[1] = force[1] - (vp[1] * fmag) / vnorm;
            force[2] = force[2] - (vp[2] * fmag) / vnorm;
        } else {
            double fp[3] = {force[0] - fn[0], force[1] - fn[1], force[2] - fn[2]};
            if (fs * nrm3(fn) > nrm3(fp)) {
                force[0] = force[0] - fp[0];
                force[1] = force[1] - fp[1];
                force[2] = force[2] - fp[2];
            }
        }
    }
    if (disp < 0) {
        double s = (-disp) * TO_NORMAL;
        force[0] = force[0] + n[0] * s;
        force[1] = force[1] + n[1] * s;
        force[2] = force[2] + n[2] * s;
    } else {
        force[0] = force[0] + n[0] * 0.0;
        force[1] = force[1] + n[1] * 0.0;
        force[2] = force[2] + n[2] * 0.0;
    }
}

/* src/object.cu:115-124. */
void to_constraint_plane_apply(const double n[3], double friction, double vel[3], double force[3]) {
    double nf = dot3(force, n);
    force[0] = force[0] + (-n[0]) * nf;
    force[1] = force[1] + (-n[1]) * nf;
    force[2] = force[2] + (-n[2]) * nf;
    double vn = nrm3(vel);
    if (vn >= 1e-16) {
        double vdn = dot3(vel, n);
        vel[0] = vel[0] + (-n[0]) * vdn;
        vel[1] = vel[1] + (-n[1]) * vdn;
        vel[2] = vel[2] + (-n[2]) * vdn;
        double s = (-friction) * nf;
        force[0] = force[0] + (vel[0] * s) / vn;
        force[1] = force[1] + (vel[1] * s) / vn;
        force[2] = force[2] + (vel[2] * s) / vn;
    }
}

/* src/object.cu:133-141. */
void to_direction_apply(const double t[3], double friction, double vel[3], double force[3]) {
    double fdt = dot3(force, t);
    double nf[3] = {force[0] - t[0] * fdt, force[1] - t[1] * fdt, force[2] - t[2] * fdt};
    force[0] = force[0] + (-nf[0]);
    force[1] = force[1] + (-nf[1]);
    force[2] = force[2] + (-nf[2]);
    if (nrm3(vel) >= 1e-16) {
        double vdt = dot3(vel, t);
        vel[0] = t[0] * vdt;
        vel[1] = t[1] * vdt;
        vel[2] = t[2] * vdt;
        double s = (-nrm3(nf)) * friction;
        force[0] = force[0] + t[0] * s;
        force[1] = force[1] + t[1] * s;
        force[2] = force[2] + t[2] * s;
    }
}

/* Per-mass part of src/sim.cu:1096-1168 (CONSTRAINTS on).  stage: RK2's
 * first (0) or second (1) half step; bx, bv: RK2 backups of this mass. */
static void mass_update(to_scene *s, int64_t i, int stage, double *bx, double *bv) {
    if (s->fixed && s->fixed[i]) return;
    double *F = s->force + 3 * i;
    double *x = s->pos + 3 * i;
    double *v = s->vel + 3 * i;
    double m = s->m[i];
    F[0] = F[0] + s->g[0] * m;
    F[1] = F[1] + s->g[1] * m;
    F[2] = F[2] + s->g[2] * m;
    if (s->ext) {
        F[0] = F[0] + s->ext[3 * i];
        F[1] = F[1] + s->ext[3 * i + 1];
        F[2] = F[2] + s->ext[3 * i + 2];
    } else {
        F[0] = F[0] + 0.0;
        F[1] = F[1] + 0.0;
        F[2] = F[2] + 0.0;
    }
    for (int32_t j = 0; j < s->n_planes; j++)
        to_plane_apply(s->plane_n + 3 * j, s->plane_off[j], s->plane_fk[j], s->plane_fs[j], x, v, F);
    for (int32_t j = 0; j < s->n_balls; j++)
        to_ball_apply(s->ball_c + 3 * j, s->ball_r[j], x, F);
    if (s->mass_bp && s->mass_bp[i] >= 0) {
        int32_t b = s->mass_bp[i];
        to_plane_apply(s->bp_n + 3 * b, s->bp_off[b], s->bp_fk[b], s->bp_fs[b], x, v, F);
    }
    if (s->lc_ptr) {
        for (int64_t r = s->lc_ptr[i]; r < s->lc_ptr[i + 1]; r++) {
            const double *vec = s->lc_vec + 3 * r;
            double num = s->lc_num[r];
            switch (s->lc_type[r]) {
                case TO_CONTACT_PLANE: to_plane_apply(vec, num, 0.0, 0.0, x, v, F); break;
                case TO_BALL: to_ball_apply(vec, num, x, F); break;
                case TO_CONSTRAINT_PLANE: to_constraint_plane_apply(vec, num, v, F); break;
                case TO_DIRECTION: to_direction_apply(vec, num, v, F); break;
                default: break;
            }
        }
    }
    double vn = nrm3(v);
    if (vn != 0.0) {
        double nv = nrm3(v);
        double c = (double)(-(s->drag ? s->drag[i] : 0)) * (nv * nv);
        F[0] = F[0] + (v[0] * c) / nv;
        F[1] = F[1] + (v[1] * c) / nv;
        F[2] = F[2] + (v[2] * c) / nv;
    }
    const double dt = s->dt;
    double a[3] = {F[0] / m, F[1] / m, F[2] / m};
    if (s->integrator == TO_VERLET) {  /* src/sim.cu:1155-1159 */
        double *ac = s->acc + 3 * i;
        const double dt2 = pow(dt, 2);
        for (int c = 0; c < 3; c++) v[c] = v[c] + (0.5 * (ac[c] + a[c])) * dt;
        for (int c = 0; c < 3; c++) ac[c] = a[c];
        for (int c = 0; c < 3; c++) x[c] = x[c] + (v[c] * dt + (0.5 * ac[c]) * dt2);
        if (s->T) s->T[i] = s->T[i] + dt;
    } else if (s->integrator == TO_RK2) {  /* src/sim.cu:1141-1154 */
        if (s->acc)
            for (int c = 0; c < 3; c++) s->acc[3 * i + c] = a[c];
        if (stage == 0) {
            for (int c = 0; c < 3; c++) {
                bv[c] = v[c];
                bx[c] = x[c];
            }
            for (int c = 0; c < 3; c++) x[c] = x[c] + (0.5 * v[c]) * dt;
            for (int c = 0; c < 3; c++) v[c] = v[c] + (0.5 * a[c]) * dt;
        } else {
            for (int c = 0; c < 3; c++) x[c] = bx[c] + v[c] * dt;
            for (int c = 0; c < 3; c++) v[c] = bv[c] + a[c] * dt;
        }
        if (s->T) s->T[i] = s->T[i] + 0.5 * dt;
    } else {  /* symplectic Euler, src/sim.cu:1161-1166 */
        if (s->acc)
            for (int c = 0; c < 3; c++) s->acc[3 * i + c] = a[c];
        v[0] = v[0] + a[0] * dt;
        v[1] = v[1] + a[1] * dt;
        v[2] = v[2] + a[2] * dt;
        x[0] = x[0] + v[0] * dt;
        x[1] = x[1] + v[1] * dt;
        x[2] = x[2] + v[2] * dt;
        if (s->T) s->T[i] = s->T[i] + dt;
    }
    F[0] = 0.0;
    F[1] = 0.0;
    F[2] = 0.0;
}

static int spring_valid(const to_scene *s, int64_t j) {
    int32_t l = s->left[j], r = s->right[j];
    return l >= 0 && r >= 0 && l < s->n_masses && r < s->n_masses;
}

static void spring_eval(const to_scene *s, int64_t j, double F[3]) {
    int32_t l = s->left[j], r = s->right[j];
    to_spring_force(s->pos + 3 * l, s->pos + 3 * r, s->vel + 3 * l, s->vel + 3 * r,
                    s->k[j], s->rest[j], s->damping[j], s->type ? s->type[j] : 0,
                    s->omega ? s->omega[j] : 0.0, s->amp ? s->amp[j] : 0.2,
                    s->phase ? s->phase[j] : 0.0, s->T_global, F);
}

static void add_to(to_scene *s, int32_t i, const double F[3], double sign) {
    if (s->fixed && s->fixed[i]) return;
    double *f = s->force + 3 * i;
    if (sign > 0) {
        f[0] = f[0] + F[0];
        f[1] = f[1] + F[1];
        f[2] = f[2] + F[2];
    } else {
        f[0] = f[0] + (-F[0]);
        f[1] = f[1] + (-F[1]);
        f[2] = f[2] + (-F[2]);
    }
}

/* Per-mass incidence lists in ascending spring order (right before left for a
 * spring attached twice to the same mass), for TO_ORDER_DEVICE. */
typedef struct { int64_t *ptr; int64_t *spring; int8_t *sign; } inc_list;

static int build_incidence(const to_scene *s, inc_list *L) {
    int64_t n = s->n_masses;
    L->ptr = (int64_t *)calloc((size_t)(n + 1), sizeof(int64_t));
    if (!L->ptr) return -1;
    for (int64_t j = 0; j < s->n_springs; j++) {
        if (!spring_valid(s, j)) continue;
        L->ptr[s->right[j] + 1]++;
        L->ptr[s->left[j] + 1]++;
    }
    for (int64_t i = 0; i < n; i++) L->ptr[i + 1] += L->ptr[i];
    int64_t tot = L->ptr[n];
    L->spring = (int64_t *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(int64_t));
    L->sign = (int8_t *)malloc((size_t)(tot > 0 ? tot : 1));
    int64_t *fill = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    if (!L->spring || !L->sign || !fill) return -1;
    memcpy(fill, L->ptr, (size_t)n * sizeof(int64_t));
    for (int64_t j = 0; j < s->n_springs; j++) {
        if (!spring_valid(s, j)) continue;
        int32_t r = s->right[j], l = s->left[j];
        L->spring[fill[r]] = j; L->sign[fill[r]] = 1; fill[r]++;
        L->spring[fill[l]] = j; L->sign[fill[l]] = -1; fill[l]++;
    }
    free(fill);
    return 0;
}

static void free_incidence(inc_list *L) {
    free(L->ptr); free(L->spring); free(L->sign);
}

int to_step(to_scene *s, int64_t nsteps, int order, int nthreads) {
    if (order < TO_ORDER_ASCENDING || order > TO_ORDER_DEVICE) return -2;
    if (s->integrator == TO_VERLET && !s->acc) return -3;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int64_t ns = s->n_springs, n = s->n_masses;
    inc_list L = {0, 0, 0};
    double *Fs = NULL;
    if (order == TO_ORDER_DEVICE) {
        if (build_incidence(s, &L) != 0) return -1;
        Fs = (double *)malloc((size_t)(ns > 0 ? ns : 1) * 3 * sizeof(double));
        if (!Fs) return -1;
    }
    double *bk = NULL;  /* RK2 backups: position and velocity per mass */
    const int passes = s->integrator == TO_RK2 ? 2 : 1;
    if (passes == 2) {
        bk = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
        if (!bk) return -1;
    }
    for (int64_t pass = 0; pass < nsteps * passes; pass++) {
        const int stage = (int)(pass % passes);
        if (order == TO_ORDER_ASCENDING) {
            for (int64_t j = 0; j < ns; j++) {
                if (!spring_valid(s, j)) continue;
                double F[3];
                spring_eval(s, j, F);
                add_to(s, s->right[j], F, 1.0);
                add_to(s, s->left[j], F, -1.0);
            }
        } else if (order == TO_ORDER_DESCENDING) {
            for (int64_t j = ns - 1; j >= 0; j--) {
                if (!spring_valid(s, j)) continue;
                double F[3];
                spring_eval(s, j, F);
                add_to(s, s->right[j], F, 1.0);
                add_to(s, s->left[j], F, -1.0);
            }
        } else if (order == TO_ORDER_ATOMIC_OMP) {
            #pragma omp parallel for schedule(static)
            for (int64_t j = 0; j < ns; j++) {
                if (!spring_valid(s, j)) continue;
                double F[3];
                spring_eval(s, j, F);
                int32_t r = s->right[j], l = s->left[j];
                if (!(s->fixed && s->fixed[r])) {
                    double *f = s->force + 3 * r;
                    #pragma omp atomic
                    f[0] += F[0];
                    #pragma omp atomic
                    f[1] += F[1];
                    #pragma omp atomic
                    f[2] += F[2];
                }
                if (!(s->fixed && s->fixed[l])) {
                    double *f = s->force + 3 * l;
                    #pragma omp atomic
                    f[0] += -F[0];
                    #pragma omp atomic
                    f[1] += -F[1];
                    #pragma omp atomic
                    f[2] += -F[2];
                }
            }
        } else if (order == TO_ORDER_DEVICE) {
            #pragma omp parallel for schedule(static)
            for (int64_t j = 0; j < ns; j++) {
                if (!spring_valid(s, j)) continue;
                spring_eval(s, j, Fs + 3 * j);
            }
            int32_t H = s->heavy_threshold > 0 ? s->heavy_threshold : 0x7fffffff;
            #pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) {
                if (s->fixed && s->fixed[i]) continue;
                int64_t b = L.ptr[i], e = L.ptr[i + 1];
                double *f = s->force + 3 * i;
                if (e - b <= H) {
                    for (int64_t q = b; q < e; q++) {
                        const double *F = Fs + 3 * L.spring[q];
                        if (L.sign[q] > 0) {
                            f[0] = f[0] + F[0]; f[1] = f[1] + F[1]; f[2] = f[2] + F[2];
                        } else {
                            f[0] = f[0] + (-F[0]); f[1] = f[1] + (-F[1]); f[2] = f[2] + (-F[2]);
                        }
                    }
                } else {
                    /* warp-cooperative order: lane l sums incidences l, l+32, ...
                       starting from +0.0, then an xor butterfly over 32 lanes. */
                    for (int c = 0; c < 3; c++) {
                        double p[32];
                        for (int l = 0; l < 32; l++) p[l] = 0.0;
                        for (int64_t q = b; q < e; q++) {
                            int l = (int)((q - b) & 31);
                            double v = Fs[3 * L.spring[q] + c];
                            p[l] = p[l] + (L.sign[q] > 0 ? v : -v);
                        }
                        for (int off = 16; off >= 1; off >>= 1)
                            for (int l = 0; l < off; l++) p[l] = p[l] + p[l + off];
                        f[c] = f[c] + p[0];
                    }
                }
            }
        }
        #pragma omp parallel for schedule(static) if (order == TO_ORDER_ATOMIC_OMP || order == TO_ORDER_DEVICE)
        for (int64_t i = 0; i < n; i++)
            mass_update(s, i, stage, bk ? bk + 6 * i : NULL, bk ? bk + 6 * i + 3 : NULL);
        s->T_global = s->T_global + (passes == 2 ? 0.5 * s->dt : s->dt);
    }
    free(bk);
    if (order == TO_ORDER_DEVICE) {
        free_incidence(&L);
        free(Fs);
    }
    return 0;
}

/* Spring count of a lattice: the builder adds, per mass, the forward
 * neighbours of the 26-neighbourhood (src/object.cu:247-288). */
int64_t to_lattice_springs(int nx, int ny, int nz) {
    int64_t cnt = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                int li = (i != nx - 1) ? 2 : 1, mj = (j != ny - 1) ? 2 : 1, nk = (k != nz - 1) ? 2 : 1;
                cnt += (int64_t)li * mj * nk - 1;
                if (k != nz - 1) {
                    if (j != ny - 1) cnt++;
                    if (i != nx - 1) cnt++;
                    if (j != ny - 1 && i != nx - 1) cnt += 3;
                }
                if (j != ny - 1 && i != nx - 1) cnt++;
            }
    return cnt;
}

/* src/object.cu:232-293: masses in i, j, k order; springs to the forward
 * neighbours in the builder's loop order; rest length = |right - left|. */
void to_lattice(const double center[3], const double dims[3], int nx, int ny, int nz,
                double *pos, int32_t *left, int32_t *right, double *rest) {
    int64_t q = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                double u = (nx > 1) ? (double)i / (nx - 1.0) - 0.5 : 0;
                double v = (ny > 1) ? j / (ny - 1.0) - 0.5 : 0;
                double w = (nz > 1) ? k / (nz - 1.0) - 0.5 : 0;
                pos[3 * q] = u * dims[0] + center[0];
                pos[3 * q + 1] = v * dims[1] + center[1];
                pos[3 * q + 2] = w * dims[2] + center[2];
                q++;
            }
#define IDX(a, b, c) ((int32_t)((c) + (b) * nz + (a) * ny * nz))
    int64_t s = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                for (int l = 0; l < ((i != nx - 1) ? 2 : 1); l++)
                    for (int m = 0; m < ((j != ny - 1) ? 2 : 1); m++)
                        for (int n = 0; n < ((k != nz - 1) ? 2 : 1); n++)
                            if (l != 0 || m != 0 || n != 0) {
                                left[s] = IDX(i, j, k);
                                right[s] = IDX(i + l, j + m, k + n);
                                s++;
                            }
                if (k != nz - 1) {
                    if (j != ny - 1) { left[s] = IDX(i, j, k + 1); right[s] = IDX(i, j + 1, k); s++; }
                    if (i != nx - 1) { left[s] = IDX(i, j, k + 1); right[s] = IDX(i + 1, j, k); s++; }
                    if (j != ny - 1 && i != nx - 1) {
                        left[s] = IDX(i, j, k + 1); right[s] = IDX(i + 1, j + 1, k); s++;
                        left[s] = IDX(i + 1, j, k + 1); right[s] = IDX(i, j + 1, k); s++;
                        left[s] = IDX(i, j + 1, k + 1); right[s] = IDX(i + 1, j, k); s++;
                    }
                }
                if (j != ny - 1 && i != nx - 1) { left[s] = IDX(i, j + 1, k); right[s] = IDX(i + 1, j, k); s++; }
            }
#undef IDX
    for (int64_t t = 0; t < s; t++) {
        const double *a = pos + 3 * left[t], *b = pos + 3 * right[t];
        double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        rest[t] = nrm3(d);
    }
}

void to_energy(const to_scene *s, double g_mag, double out[4]) {
    double pg = 0, ke = 0, ps = 0;
    for (int64_t i = 0; i < s->n_masses; i++) {
        double m = s->m[i];
        pg = pg + (g_mag * s->pos[3 * i + 2]) * m;
        double vn = nrm3(s->vel + 3 * i);
        ke = ke + (0.5 * m) * (vn * vn);
    }
    for (int64_t j = 0; j < s->n_springs; j++) {
        if (!spring_valid(s, j)) continue;
        const double *a = s->pos + 3 * s->left[j], *b = s->pos + 3 * s->right[j];
        double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
        double x = nrm3(d) - s->rest[j];
        ps = ps + (s->k[j] * (x * x)) / 2;
    }
    out[0] = ps;
    out[1] = ke;
    out[2] = pg;
    out[3] = (ps + ke) + pg;
}

void to_momentum(const to_scene *s, double lin[3], double ang[3]) {
    lin[0] = lin[1] = lin[2] = 0;
    ang[0] = ang[1] = ang[2] = 0;
    for (int64_t i = 0; i < s->n_masses; i++) {
        double m = s->m[i];
        const double *v = s->vel + 3 * i, *x = s->pos + 3 * i;
        double p[3] = {v[0] * m, v[1] * m, v[2] * m};
        lin[0] = lin[0] + p[0]; lin[1] = lin[1] + p[1]; lin[2] = lin[2] + p[2];
        ang[0] = ang[0] + (p[1] * x[2] - p[2] * x[1]);
        ang[1] = ang[1] + (x[0] * p[2] - p[0] * x[2]);
        ang[2] = ang[2] + (p[0] * x[1] - p[1] * x[0]);
    }
}

/* ---- STL point-in-mesh (include/Titan/stlparser.h:213-276) --------------- */

static uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

static double ray_component(uint64_t seed, int64_t point, int ray, int c) {
    const uint64_t k = splitmix64(seed ^ splitmix64((uint64_t)point * 3ULL * 64ULL + (uint64_t)ray * 3ULL + (uint64_t)c));
    const double u = (double)(k >> 11) * (1.0 / 9007199254740992.0);
    return -1000.0 + u * 2000.0;
}

static double sdot(const double *a, const double *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static void scross(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = b[0] * a[2] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

static int ray_hits(const double *p, const double *ray, const double *t) {
    const double eps = 0.000001;
    const double e1[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]};
    const double e2[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
    double h[3], q[3];
    scross(ray, e2, h);
    const double a = sdot(e1, h);
    if (a > -eps && a < eps) return 0;
    const double f = 1 / a;
    const double s[3] = {p[0] - t[0], p[1] - t[1], p[2] - t[2]};
    const double u = f * sdot(s, h);
    if (u < 0 || u > 1.0) return 0;
    scross(s, e1, q);
    const double v = f * sdot(ray, q);
    if (v < 0 || u + v > 1.0) return 0;
    return f * sdot(e2, q) > eps;
}

int to_stl_inside(const double *tri, int64_t ntri, const double *pts, int64_t npts, int num_rays, uint64_t seed,
                  uint8_t *inside, int nthreads) {
    if (num_rays < 1 || num_rays > 64) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    #pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < npts; i++) {
        int odd = 0;
        for (int r = 0; r < num_rays; r++) {
            double d[3];
            for (int c = 0; c < 3; c++) d[c] = ray_component(seed, i, r, c);
            const double n = sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
            const double ray[3] = {d[0] / n, d[1] / n, d[2] / n};
            int par = 0;
            for (int64_t t = 0; t < ntri; t++) par ^= ray_hits(pts + 3 * i, ray, tri + 9 * t);
            odd += par;
        }
        inside[i] = (double)odd / (double)num_rays > 0.5 ? 1 : 0;
    }
    return 0;
}

