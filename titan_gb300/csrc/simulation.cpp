// simulation.cpp -- titan::Simulation (include/Titan/sim.h) over the C ABI.
//
// Mirrors the reference's control semantics (src/sim.cu:1349-1657): start()
// uploads and runs until a breakpoint; pause(t) sets a breakpoint at
// simulated time t and blocks until it is reached; wait(t) sleeps while the
// simulation advances by t; resume() continues; stop() ends the run.  The
// reference's GPU thread (src/sim.cu:1389) becomes a request loop that runs
// CUDA-graph chunks between breakpoints and yields to get/set between chunks.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <cstdlib>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>

#include "Titan/sim.h"
#include "titan_gb300.h"

namespace titan {

namespace {
constexpr int64_t kLoopChunk = 128;  // steps between request-loop turns
const char *kEnded = "The simulation has ended. Cannot modify simulation after the end of the simulation.";
const char *kRunning = "The simulation is running. Stop the simulation to make changes.";
}  // namespace

// ---------------------------------------------------------------- Mass -----
Mass::Mass() : m(1.0), T(0.0) {}
Mass::Mass(const Vec &position, double mass, bool) : m(mass), T(0.0), pos(position) {}

void Mass::addConstraint(CONSTRAINT_TYPE type, const Vec &vec, double num) {
    constraints.push_back(LocalConstraint{type, vec, num});
}
void Mass::clearConstraints(CONSTRAINT_TYPE type) {
    constraints.erase(std::remove_if(constraints.begin(), constraints.end(),
                                     [&](const LocalConstraint &c) { return c.type == type; }),
                      constraints.end());
}
void Mass::clearConstraints() { constraints.clear(); }
void Mass::setDrag(double C) { drag_coefficient = C; }
void Mass::fix() { fixed = true; }
void Mass::unfix() { fixed = false; }
void Mass::decrementRefCount() { --ref_count; }

// -------------------------------------------------------------- Spring -----
void Spring::setLeft(Mass *left) {
    if (_left) _left->decrementRefCount();
    _left = left;
    _left->ref_count++;
}
void Spring::setRight(Mass *right) {
    if (_right) _right->decrementRefCount();
    _right = right;
    _right->ref_count++;
}

// ----------------------------------------------------------- Containers ----
void Container::translate(const Vec &displ) {
    for (Mass *m : masses) m->pos += displ;
}

// src/object.cu:198-230
void Container::rotate(const Vec &axis, double angle) {
    Vec com(0, 0, 0);
    double total = 0;
    for (Mass *m : masses) {
        com += m->m * m->pos;
        total += m->m;
    }
    com = com / total;
    Vec ax = axis / axis.norm();
    for (Mass *m : masses) {
        Vec t = m->pos - com;
        Vec y = t - dot(t, ax) * ax;
        if (y.norm() < 0.0001) continue;
        Vec planar(-std::sin(angle) * y.norm(), std::cos(angle) * y.norm(), 0);
        Vec spatial = planar[0] * cross(ax, y / y.norm()) + y / y.norm() * planar[1] + dot(t, ax) * ax + com;
        m->pos = spatial;
    }
}

void Container::setMassValues(double m) {
    for (Mass *mass : masses) mass->m += m;
}
void Container::setSpringConstants(double k) {
    for (Spring *s : springs) s->_k = k;
}
void Container::setRestLengths(double len) {
    for (Spring *s : springs) s->_rest = len;
}
void Container::addConstraint(CONSTRAINT_TYPE type, const Vec &v, double d) {
    for (Mass *m : masses) m->addConstraint(type, v, d);
}
void Container::clearConstraints() {
    for (Mass *m : masses) m->clearConstraints();
}
void Container::fix() {
    for (Mass *m : masses) m->fix();
}
void Container::add(Mass *m) { masses.push_back(m); }
void Container::add(Spring *s) { springs.push_back(s); }
void Container::add(Container *c) {
    masses.insert(masses.end(), c->masses.begin(), c->masses.end());
    springs.insert(springs.end(), c->springs.begin(), c->springs.end());
}

Cube::Cube(const Vec &center, double side_length) : _side_length(side_length), _center(center) {
    for (int i = 0; i < 8; i++)
        masses.push_back(new Mass(side_length * (Vec(i & 1, (i >> 1) & 1, (i >> 2) & 1) - Vec(0.5, 0.5, 0.5)) + center));
    for (int i = 0; i < 8; i++)
        for (int j = i + 1; j < 8; j++) springs.push_back(new Spring(masses[i], masses[j]));
    for (Spring *s : springs) s->setRestLength((s->_right->pos - s->_left->pos).norm());
}

namespace {
void build_lattice(Container &c, const Vec &center, const Vec &dims, int nx, int ny, int nz, bool fix_face) {
    int64_t n = (int64_t)nx * ny * nz;
    int64_t ns = titan_gb300_lattice_springs(nx, ny, nz);
    std::vector<double> pos(3 * n);
    std::vector<int32_t> l(ns), r(ns);
    double cc[3] = {center[0], center[1], center[2]}, dd[3] = {dims[0], dims[1], dims[2]};
    titan_gb300_lattice(cc, dd, nx, ny, nz, pos.data(), l.data(), r.data(), nullptr);
    for (int64_t i = 0; i < n; i++) {
        Mass *m = new Mass(Vec(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
        if (fix_face && i < (int64_t)ny * nz) m->fix();  // i == 0 face (src/object.cu:307-309)
        c.masses.push_back(m);
    }
    for (int64_t s = 0; s < ns; s++) c.springs.push_back(new Spring(c.masses[l[s]], c.masses[r[s]]));
    for (Spring *s : c.springs) s->setRestLength((s->_right->pos - s->_left->pos).norm());
}
}  // namespace

Lattice::Lattice(const Vec &center, const Vec &dims, int nx_, int ny_, int nz_)
    : nx(nx_), ny(ny_), nz(nz_), _center(center), _dims(dims) {
    build_lattice(*this, center, dims, nx, ny, nz, false);
}

Beam::Beam(const Vec &center, const Vec &dims, int nx_, int ny_, int nz_)
    : nx(nx_), ny(ny_), nz(nz_), _center(center), _dims(dims) {
    build_lattice(*this, center, dims, nx, ny, nz, true);
}

// ---------------------------------------------------------- Simulation -----
Simulation::Simulation() : dt(0.0001), _global_acc(0, 0, -9.81) {
    const char *p = std::getenv("TITAN_GB300_PRECISION");
    if (p) precision_ = std::atoi(p);
}

Simulation::~Simulation() {
    if (STARTED && !FREED) {
        {
            std::lock_guard<std::mutex> lk(mu);
            ENDED = true;
        }
        cv.notify_all();
        if (gpu_thread.joinable()) gpu_thread.join();
    }
    if (handle) titan_gb300_destroy(handle);
    handle = nullptr;
    for (Spring *s : springs) delete s;
    for (Spring *s : spring_graveyard) delete s;
    for (Mass *m : masses) delete m;
    for (Mass *m : graveyard) delete m;
    for (Container *c : containers) delete c;
}

void Simulation::check(int rc, const char *what) {
    if (rc != TITAN_GB300_OK)
        throw std::runtime_error(std::string(what) + ": " + titan_gb300_last_error(handle));
}

void Simulation::requireStarted(const char *) {
    if (ENDED) throw std::runtime_error(kEnded);
}

Mass *Simulation::createMass(Mass *m) {
    if (ENDED) throw std::runtime_error(kEnded);
    if (STARTED && RUNNING) throw std::runtime_error(kRunning);
    m->ref_count++;
    std::lock_guard<std::mutex> lk(mu);
    masses.push_back(m);
    if (STARTED) dirty = true;
    return m;
}
Mass *Simulation::createMass() { return createMass(new Mass()); }
Mass *Simulation::createMass(const Vec &pos) { return createMass(new Mass(pos)); }

Spring *Simulation::createSpring(Spring *s) {
    if (ENDED) throw std::runtime_error(kEnded);
    if (STARTED && RUNNING) throw std::runtime_error(kRunning);
    if (s->_right) s->_right->ref_count++;
    if (s->_left) s->_left->ref_count++;
    std::lock_guard<std::mutex> lk(mu);
    springs.push_back(s);
    if (STARTED) dirty = true;
    return s;
}
Spring *Simulation::createSpring() { return createSpring(new Spring()); }
Spring *Simulation::createSpring(Mass *m1, Mass *m2) { return createSpring(new Spring(m1, m2)); }

void Simulation::deleteMass(Mass *m) {
    if (ENDED) throw std::runtime_error(kEnded);
    if (STARTED && RUNNING) throw std::runtime_error(kRunning);
    std::lock_guard<std::mutex> lk(mu);
    masses.erase(std::remove(masses.begin(), masses.end(), m), masses.end());
    m->valid = false;
    graveyard.push_back(m);  // springs may still point at it; they are skipped
    if (STARTED) dirty = true;
}

void Simulation::deleteSpring(Spring *s) {
    if (ENDED) throw std::runtime_error(kEnded);
    if (STARTED && RUNNING) throw std::runtime_error(kRunning);
    std::lock_guard<std::mutex> lk(mu);
    springs.erase(std::remove(springs.begin(), springs.end(), s), springs.end());
    if (s->_left) s->_left->decrementRefCount();
    if (s->_right) s->_right->decrementRefCount();
    spring_graveyard.push_back(s);
    if (STARTED) dirty = true;
}

Container *Simulation::createContainer() {
    Container *c = new Container();
    containers.push_back(c);
    return c;
}

void Simulation::deleteContainer(Container *c) {
    if (ENDED) throw std::runtime_error(kEnded);
    if (RUNNING) throw std::runtime_error(kRunning);
    for (Mass *m : c->masses) deleteMass(m);
    for (Spring *s : c->springs) deleteSpring(s);
    c->masses.clear();
    c->springs.clear();
    containers.erase(std::remove(containers.begin(), containers.end(), c), containers.end());
    delete c;
}

Cube *Simulation::createCube(const Vec &center, double side_length) {
    if (ENDED) throw std::runtime_error("The simulation has ended. Cannot create new objects");
    Cube *c = new Cube(center, side_length);
    for (Mass *m : c->masses) createMass(m);
    for (Spring *s : c->springs) createSpring(s);
    containers.push_back(c);
    return c;
}

Lattice *Simulation::createLattice(const Vec &center, const Vec &dims, int nx, int ny, int nz) {
    if (ENDED) throw std::runtime_error("The simulation has ended. New objects cannot be created.");
    Lattice *l = new Lattice(center, dims, nx, ny, nz);
    masses.reserve(masses.size() + l->masses.size());
    springs.reserve(springs.size() + l->springs.size());
    for (Mass *m : l->masses) createMass(m);
    for (Spring *s : l->springs) createSpring(s);
    containers.push_back(l);
    return l;
}

Beam *Simulation::createBeam(const Vec &center, const Vec &dims, int nx, int ny, int nz) {
    if (ENDED) throw std::runtime_error("The simulation has ended. New objects cannot be created.");
    Beam *b = new Beam(center, dims, nx, ny, nz);
    for (Mass *m : b->masses) createMass(m);
    for (Spring *s : b->springs) createSpring(s);
    containers.push_back(b);
    return b;
}

// Seed of the point-in-mesh rays (the reference draws them with rand()).
constexpr uint64_t kStlSeed = 0x7469746e53544cULL;

// Simulation::importFromSTL, src/sim.cu:1855-1921: a num_pts^3 lattice over
// the mesh's bounding box, scaled so that its longest side is 10, keeps the
// masses whose point the mesh contains (titan_gb300_stl_inside, on the GPU)
// and the springs between kept masses.  Binary STL as the reference parses it
// (include/Titan/stlparser.h:300-333): an 80-byte header, a uint32 count,
// then per triangle 12 little-endian floats (normal, v1, v2, v3) and a
// 2-byte attribute.
Container *Simulation::importFromSTL(const std::string &path, double density, int num_rays) {
    if (ENDED) throw std::runtime_error("The simulation has ended. Cannot import new STL objects");
    std::ifstream f(path.c_str(), std::ios::in | std::ios::binary);
    if (!f) throw std::runtime_error("importFromSTL: cannot read " + path);
    char header[80];
    unsigned char cnt[4];
    f.read(header, 80);
    f.read(reinterpret_cast<char *>(cnt), 4);
    if (!f) throw std::runtime_error("importFromSTL: " + path + " is not a binary STL file");
    const uint32_t ntri = (uint32_t)cnt[0] | ((uint32_t)cnt[1] << 8) | ((uint32_t)cnt[2] << 16) | ((uint32_t)cnt[3] << 24);
    std::vector<double> tri(9 * (size_t)ntri);
    for (uint32_t t = 0; t < ntri; t++) {
        unsigned char rec[50];
        f.read(reinterpret_cast<char *>(rec), 50);
        if (!f) throw std::runtime_error("importFromSTL: " + path + " is truncated");
        for (int k = 0; k < 9; k++) {
            const unsigned char *b = rec + 12 + 4 * k;
            const uint32_t bits = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
            float v;
            std::memcpy(&v, &bits, 4);
            tri[9 * (size_t)t + k] = v;
        }
    }
    // bounding box as stlFile::getBoundingBox computes it (stlparser.h:193-210),
    // including its starting values {DBL_MIN, 0, 0} for both corners
    double mn[3] = {DBL_MIN, 0.0, 0.0}, mx[3] = {DBL_MIN, 0.0, 0.0};
    for (size_t q = 0; q < tri.size(); q += 3)
        for (int i = 0; i < 3; i++) {
            mn[i] = std::fmin(tri[q + i], mn[i]);
            mx[i] = std::fmax(tri[q + i], mx[i]);
        }
    const double center[3] = {(mx[0] - mn[0]) / 2 + mn[0], (mx[1] - mn[1]) / 2 + mn[1], (mx[2] - mn[2]) / 2 + mn[2]};
    const double xdim = mx[0] - mn[0], ydim = mx[1] - mn[1], zdim = mx[2] - mn[2];
    const double dimmax = std::max(std::max(xdim, ydim), zdim);
    const double dimx = 10 * xdim / dimmax, dimy = 10 * ydim / dimmax, dimz = 10 * zdim / dimmax;
    const int num_pts = (int)std::cbrt(density * std::pow(10 / dimmax, 3) * xdim * ydim * zdim);
    if (!(num_pts >= 2)) throw std::runtime_error("importFromSTL: density gives fewer than 2 lattice points per side");
    Lattice *l1 = new Lattice(Vec(0, 0, dimz), Vec(dimx - 0.001, dimy - 0.001, dimz - 0.001), num_pts, num_pts,
                              num_pts);
    const size_t n = l1->masses.size();
    std::vector<double> pts(3 * n);
    for (size_t i = 0; i < n; i++) {
        const Mass *m = l1->masses[i];
        pts[3 * i] = center[0] + (xdim / dimx) * m->pos[0];
        pts[3 * i + 1] = center[1] + (ydim / dimy) * m->pos[1];
        pts[3 * i + 2] = (zdim / dimz) * (m->pos[2] - dimz) + center[2];
    }
    std::vector<uint8_t> in(n, 0);
    const int rc = titan_gb300_stl_inside(0, tri.data(), (int64_t)ntri, pts.data(), (int64_t)n, num_rays, kStlSeed,
                                          in.data());
    if (rc != TITAN_GB300_OK) {
        delete l1;
        throw std::runtime_error("importFromSTL: the point-in-mesh test failed (status " + std::to_string(rc) + ")");
    }
    std::unordered_map<const Mass *, bool> keep;
    for (size_t i = 0; i < n; i++) keep[l1->masses[i]] = in[i] != 0;
    std::vector<Spring *> springs_kept;
    for (Spring *sp : l1->springs) {
        if (keep[sp->_left] && keep[sp->_right])
            springs_kept.push_back(sp);
        else
            delete sp;
    }
    std::vector<Mass *> masses_kept;
    for (Mass *m : l1->masses) {
        if (keep[m])
            masses_kept.push_back(m);
        else
            delete m;
    }
    l1->springs = springs_kept;
    l1->masses = masses_kept;
    masses.reserve(masses.size() + l1->masses.size());
    springs.reserve(springs.size() + l1->springs.size());
    for (Mass *m : l1->masses) createMass(m);
    for (Spring *sp : l1->springs) createSpring(sp);
    containers.push_back(l1);
    return l1;
}

void Simulation::createPlane(const Vec &abc, double d) { createPlane(abc, d, 0.0, 0.0); }

void Simulation::createPlane(const Vec &abc, double d, double FRICTION_K, double FRICTION_S) {
    if (ENDED) throw std::runtime_error("The simulation has ended. New objects cannot be created.");
    std::lock_guard<std::mutex> lk(mu);
    planes.push_back(Plane{abc, d, FRICTION_K, FRICTION_S});
    if (handle) {
        double n[3] = {abc[0], abc[1], abc[2]};
        check(titan_gb300_add_plane(handle, n, d, FRICTION_K, FRICTION_S), "createPlane");
    }
}

void Simulation::createBall(const Vec &center, double r) {
    if (ENDED) throw std::runtime_error("The simulation has ended. New constraints cannot be added.");
    std::lock_guard<std::mutex> lk(mu);
    balls.push_back(Ball{center, r});
    if (handle) {
        double c[3] = {center[0], center[1], center[2]};
        check(titan_gb300_add_ball(handle, c, r), "createBall");
    }
}

void Simulation::clearConstraints() {
    std::lock_guard<std::mutex> lk(mu);
    planes.clear();
    balls.clear();
    if (handle) check(titan_gb300_clear_constraints(handle), "clearConstraints");
}

void Simulation::setAllSpringConstantValues(double k) {
    if (ENDED) throw std::runtime_error(kEnded);
    for (Spring *s : springs) s->_k = k;
}
void Simulation::defaultRestLengths() {
    if (ENDED) throw std::runtime_error(kEnded);
    for (Spring *s : springs) s->defaultLength();
}
void Simulation::setAllMassValues(double m) {
    if (ENDED) throw std::runtime_error(kEnded);
    for (Mass *mass : masses) mass->m += m;
}
void Simulation::setTimeStep(double delta_t) {
    if (ENDED) throw std::runtime_error(kEnded);
    if (delta_t <= 0) throw std::runtime_error("Cannot set time step to negative or zero value.");
    std::lock_guard<std::mutex> lk(mu);
    dt = delta_t;
    if (handle) check(titan_gb300_set_time_step(handle, delta_t), "setTimeStep");
}
double Simulation::getTimeStep() { return dt; }

void Simulation::setGlobalAcceleration(const Vec &global_acc) {
    if (RUNNING) throw std::runtime_error("The simulation is running. The global force parameter cannot be changed during runtime");
    std::lock_guard<std::mutex> lk(mu);
    _global_acc = global_acc;
    if (handle) {
        double g[3] = {global_acc[0], global_acc[1], global_acc[2]};
        check(titan_gb300_set_global_acc(handle, g), "setGlobalAcceleration");
    }
}

void Simulation::setPrecision(int p) {
    if (STARTED) throw std::runtime_error("setPrecision must be called before start()");
    if (p < 0 || p > 2) throw std::runtime_error("precision must be 0 (FP64), 1 (FP32) or 2 (FP32C)");
    precision_ = p;
}

// Uploads the whole scene.  With keep_device_state, masses that were already
// on the device keep their device position/velocity/time (the host copies of
// those may be stale, as in the reference until get()).  Caller holds mu.
void Simulation::buildDevice(bool keep_device_state) {
    const int64_t n = (int64_t)masses.size();
    std::vector<double> dpos, dvel, dT;
    std::unordered_map<Mass *, int64_t> old_index;
    if (keep_device_state && handle) {
        int64_t on = (int64_t)built_masses.size();
        dpos.resize(3 * on);
        dvel.resize(3 * on);
        dT.resize(on);
        check(titan_gb300_get_state(handle, dpos.data(), dvel.data(), nullptr, dT.data()), "rebuild");
        for (int64_t i = 0; i < on; i++) old_index[built_masses[i]] = i;
    }
    double Tnow = T.load();
    if (handle) steps_base += (long)titan_gb300_steps(handle);
    if (handle) titan_gb300_destroy(handle);
    handle = nullptr;
    titan_gb300_sim *h = nullptr;
    int rc = titan_gb300_create(&h, 0, precision_);
    if (rc) throw std::runtime_error("titan_gb300_create failed");
    handle = h;
    std::vector<double> pos(3 * n), vel(3 * n), m(n), ext(3 * n), drag(n), mT(n);
    std::vector<uint8_t> fixed(n);
    std::vector<int64_t> lc_ptr(n + 1, 0);
    std::vector<int32_t> lc_type;
    std::vector<double> lc_vec, lc_num;
    std::unordered_map<Mass *, int32_t> index;
    for (int64_t i = 0; i < n; i++) {
        Mass *ms = masses[i];
        index[ms] = (int32_t)i;
        ms->index = i;
        auto it = old_index.find(ms);
        for (int c = 0; c < 3; c++) {
            pos[3 * i + c] = it != old_index.end() ? dpos[3 * it->second + c] : ms->pos[c];
            vel[3 * i + c] = it != old_index.end() ? dvel[3 * it->second + c] : ms->vel[c];
            ext[3 * i + c] = ms->extern_force[c];
        }
        mT[i] = it != old_index.end() ? dT[it->second] : ms->T;
        m[i] = ms->m;
        fixed[i] = ms->fixed ? 1 : 0;
        drag[i] = ms->drag_coefficient;
        for (const LocalConstraint &lc : ms->constraints) {
            lc_type.push_back((int32_t)lc.type);
            for (int c = 0; c < 3; c++) lc_vec.push_back(lc.vec[c]);
            lc_num.push_back(lc.num);
        }
        lc_ptr[i + 1] = (int64_t)lc_type.size();
    }
    const int64_t ns = (int64_t)springs.size();
    std::vector<int32_t> l(ns), r(ns), ty(ns);
    std::vector<double> k(ns), rest(ns), damp(ns), om(ns), amp(ns), ph(ns);
    for (int64_t j = 0; j < ns; j++) {
        Spring *s = springs[j];
        s->index = j;
        auto li = s->_left ? index.find(s->_left) : index.end();
        auto ri = s->_right ? index.find(s->_right) : index.end();
        l[j] = li != index.end() && s->_left->valid ? li->second : -1;
        r[j] = ri != index.end() && s->_right->valid ? ri->second : -1;
        k[j] = s->_k;
        rest[j] = s->_rest;
        damp[j] = s->_damping;
        ty[j] = (int32_t)s->_type;
        om[j] = s->_omega;
        amp[j] = s->_amplitude;
        ph[j] = s->_phase;
    }
    check(titan_gb300_set_time_step(handle, dt), "setTimeStep");
    double g[3] = {_global_acc[0], _global_acc[1], _global_acc[2]};
    check(titan_gb300_set_global_acc(handle, g), "setGlobalAcceleration");
    check(titan_gb300_set_masses(handle, n, pos.data(), vel.data(), m.data(), ext.data(), fixed.data(), drag.data()),
          "masses");
    check(titan_gb300_set_springs(handle, ns, l.data(), r.data(), k.data(), rest.data(), damp.data(), ty.data(),
                                  om.data(), amp.data(), ph.data()),
          "springs");
    if (!lc_type.empty())
        check(titan_gb300_set_local_constraints(handle, lc_ptr.data(), lc_type.data(), lc_vec.data(), lc_num.data()),
              "constraints");
    for (const Plane &p : planes) {
        double nn[3] = {p.n[0], p.n[1], p.n[2]};
        check(titan_gb300_add_plane(handle, nn, p.d, p.fk, p.fs), "createPlane");
    }
    for (const Ball &b : balls) {
        double c[3] = {b.c[0], b.c[1], b.c[2]};
        check(titan_gb300_add_ball(handle, c, b.r), "createBall");
    }
    check(titan_gb300_start(handle, 0), "start");
    if (Tnow != 0.0) check(titan_gb300_set_time(handle, Tnow), "time");
    bool anyT = false;
    for (double t : mT) anyT = anyT || t != 0.0;
    if (anyT)
        check(titan_gb300_set_mass_state(handle, n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                         mT.data()),
              "mass time");
    built_masses = masses;
    built_springs = springs;
    built_ends.resize(ns);
    for (int64_t j = 0; j < ns; j++) built_ends[j] = {springs[j]->_left, springs[j]->_right};
    dirty = false;
}

void Simulation::syncTopology() {
    if (dirty) buildDevice(true);
}

void Simulation::start() {
    if (ENDED) throw std::runtime_error("The simulation has ended. Cannot call sim.start() after the end of the simulation.");
    if (masses.empty()) throw std::runtime_error("No masses have been added. Please add masses before starting the simulation.");
    if (dt <= 0) throw std::runtime_error("Simultation timestep Simulation::dt is invalid. Please choose a positive non-zero value.");
    std::cout << "Starting simulation with " << masses.size() << " masses and " << springs.size() << " springs." << std::endl;
    {
        std::lock_guard<std::mutex> lk(mu);
        T = 0.0;
        buildDevice(false);
        RUNNING = true;
        STARTED = true;
    }
    gpu_thread = std::thread(&Simulation::loop, this);
}

// The request loop: one turn = breakpoint check + one chunk of steps.
void Simulation::loop() {
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        cv.wait(lk, [&] { return ENDED.load() || RUNNING.load(); });
        if (ENDED) break;
        syncTopology();
        double t = titan_gb300_time(handle);
        if (!bpts.empty() && *bpts.begin() <= t) {  // src/sim.cu:1505-1511
            bpts.erase(bpts.begin());
            RUNNING = false;
            cv.notify_all();
            continue;
        }
        int64_t nsteps = kLoopChunk;
        if (!bpts.empty()) {
            double bp = *bpts.begin(), tt = t;
            int64_t k = 0;
            while (tt < bp && k < kLoopChunk) {
                tt = tt + dt;
                k++;
            }
            nsteps = k;
        }
        int rc = titan_gb300_step(handle, nsteps);
        if (rc == TITAN_GB300_OK) rc = titan_gb300_synchronize(handle);
        if (rc != TITAN_GB300_OK) {
            std::cerr << "titan_gb300: " << titan_gb300_last_error(handle) << std::endl;
            RUNNING = false;
            cv.notify_all();
            continue;
        }
        T = titan_gb300_time(handle);
        // let get/set/pause in other threads take the lock between chunks
        lk.unlock();
        std::this_thread::yield();
        lk.lock();
    }
    GPU_DONE = true;
}

void Simulation::setBreakpoint(double time) {
    if (ENDED) throw std::runtime_error("The simulation has ended. Cannot set breakpoints after the end of the simulation run.");
    std::lock_guard<std::mutex> lk(mu);
    bpts.insert(time);
}

void Simulation::waitForEvent() {
    if (ENDED && !FREED) throw std::runtime_error("The simulation has ended. Control functions cannot be called.");
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return !RUNNING.load(); });
}

void Simulation::pause(double t) {
    if (ENDED) throw std::runtime_error("The simulation has ended. Control functions cannot be called.");
    setBreakpoint(t);
    waitForEvent();
}

void Simulation::wait(double t) {
    if (ENDED) throw std::runtime_error("The simulation has ended. Control functions cannot be called.");
    double current = time();
    while (RUNNING && time() <= current + t) std::this_thread::sleep_for(std::chrono::microseconds(10));
}

void Simulation::waitUntil(double t) {
    if (ENDED && !FREED) throw std::runtime_error("The simulation has ended. Control functions cannot be called.");
    while (RUNNING && time() <= t) std::this_thread::sleep_for(std::chrono::microseconds(10));
}

void Simulation::resume() {
    if (ENDED) throw std::runtime_error("The simulation has ended. Cannot resume the simulation.");
    if (!STARTED) throw std::runtime_error("The simulation has not started. You cannot resume a simulation before calling sim.start().");
    if (masses.empty()) throw std::runtime_error("No masses have been added. Please add masses before starting the simulation.");
    {
        std::lock_guard<std::mutex> lk(mu);
        RUNNING = true;
    }
    cv.notify_all();
}

void Simulation::stop() {
    if (RUNNING) {
        setBreakpoint(time());
        waitForEvent();
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        ENDED = true;
    }
    cv.notify_all();
    if (gpu_thread.joinable()) gpu_thread.join();
    if (handle) titan_gb300_destroy(handle);
    handle = nullptr;
    FREED = true;
}

void Simulation::stop(double t) {
    if (RUNNING) {
        setBreakpoint(t);
        waitForEvent();
    }
    stop();
}

void Simulation::reset() {
    if (RUNNING) throw std::runtime_error(kRunning);
    masses.clear();
    springs.clear();
    containers.clear();
    planes.clear();
    balls.clear();
    bpts.clear();
    _global_acc = Vec(0, 0, -9.81);
}

double Simulation::time() { return T.load(); }
bool Simulation::running() { return RUNNING.load(); }

void Simulation::step(long n) {
    if (!STARTED || ENDED) throw std::runtime_error("step() needs a started simulation");
    if (RUNNING) throw std::runtime_error(kRunning);
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    check(titan_gb300_step(handle, n), "step");
    check(titan_gb300_synchronize(handle), "step");
    T = titan_gb300_time(handle);
}

long Simulation::steps() { return steps_base + (handle ? (long)titan_gb300_steps(handle) : 0); }

void Simulation::diagnostics(double g_mag, double energy[4], double momentum[6]) {
    if (!STARTED || ENDED) throw std::runtime_error("diagnostics needs a started simulation");
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    check(titan_gb300_diagnostics(handle, g_mag, energy, momentum), "diagnostics");
}

// ----------------------------------------------------------- get / set -----
void Simulation::get(Mass *m) {
    if (!STARTED) {
        std::cerr << "The simulation has not started. Get and set commands cannot be called before sim.start()" << std::endl;
        return;
    }
    if (ENDED) throw std::runtime_error(kEnded);
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    int64_t idx = m->index;
    double p[3], v[3], a[3], t;
    check(titan_gb300_get_masses(handle, 1, &idx, p, v, a, &t), "get");
    m->pos = Vec(p[0], p[1], p[2]);
    m->vel = Vec(v[0], v[1], v[2]);
    m->acc = Vec(a[0], a[1], a[2]);
    m->T = t;
}

void Simulation::set(Mass *m) {
    if (!STARTED) {
        std::cerr << "The simulation has not started. Get and set commands cannot be called before sim.start()" << std::endl;
        return;
    }
    if (ENDED) throw std::runtime_error(kEnded);
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    int64_t idx = m->index;
    double p[3] = {m->pos[0], m->pos[1], m->pos[2]}, v[3] = {m->vel[0], m->vel[1], m->vel[2]};
    double e[3] = {m->extern_force[0], m->extern_force[1], m->extern_force[2]};
    double mm = m->m, dr = m->drag_coefficient, t = m->T;
    uint8_t fx = m->fixed ? 1 : 0;
    check(titan_gb300_set_mass_state(handle, 1, &idx, p, v, &mm, e, &fx, &dr, &t), "set");
}

void Simulation::get(Spring *) {
    if (!STARTED) {
        std::cerr << "The simulation has not started. Get and set commands cannot be called before sim.start()" << std::endl;
        return;
    }
    if (ENDED) throw std::runtime_error(kEnded);
    // springs are never changed by the step (src/spring.cu:12)
}

void Simulation::set(Spring *s) {
    if (!STARTED) {
        std::cerr << "The simulation has not started. Get and set commands cannot be called before sim.start()" << std::endl;
        return;
    }
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    int64_t j = s->index;
    if (j < 0 || j >= (int64_t)built_springs.size() || built_springs[j] != s) return;
    // an endpoint change is a topology change: rebuild, keeping device state
    if (built_ends[j].first != s->_left || built_ends[j].second != s->_right) {
        dirty = true;
        syncTopology();
        return;
    }
    int32_t ty = (int32_t)s->_type;
    check(titan_gb300_set_spring_params(handle, 1, &j, &s->_k, &s->_rest, &s->_damping, &ty, &s->_omega,
                                        &s->_amplitude, &s->_phase),
          "set");
}

void Simulation::getAll() {
    if (!STARTED) {
        std::cerr << "The simulation has not started. Get and set commands cannot be called before sim.start()" << std::endl;
        return;
    }
    if (ENDED) throw std::runtime_error(kEnded);
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    const int64_t n = (int64_t)masses.size();
    std::vector<double> p(3 * n), v(3 * n), a(3 * n), t(n);
    check(titan_gb300_get_state(handle, p.data(), v.data(), a.data(), t.data()), "getAll");
    for (int64_t i = 0; i < n; i++) {
        Mass *m = masses[i];
        m->pos = Vec(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
        m->vel = Vec(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        m->acc = Vec(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
        m->T = t[i];
    }
}

void Simulation::setAll() {
    if (ENDED) throw std::runtime_error(kEnded);
    if (!STARTED) return;
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    const int64_t n = (int64_t)masses.size();
    std::vector<double> p(3 * n), v(3 * n), m(n), e(3 * n), dr(n), t(n);
    std::vector<uint8_t> fx(n);
    for (int64_t i = 0; i < n; i++) {
        Mass *ms = masses[i];
        for (int c = 0; c < 3; c++) {
            p[3 * i + c] = ms->pos[c];
            v[3 * i + c] = ms->vel[c];
            e[3 * i + c] = ms->extern_force[c];
        }
        m[i] = ms->m;
        dr[i] = ms->drag_coefficient;
        t[i] = ms->T;
        fx[i] = ms->fixed ? 1 : 0;
    }
    check(titan_gb300_set_mass_state(handle, n, nullptr, p.data(), v.data(), m.data(), e.data(), fx.data(), dr.data(),
                                     t.data()),
          "setAll");
    const int64_t ns = (int64_t)springs.size();
    std::vector<double> k(ns), rest(ns), damp(ns), om(ns), amp(ns), ph(ns);
    std::vector<int32_t> ty(ns);
    for (int64_t j = 0; j < ns; j++) {
        Spring *s = springs[j];
        k[j] = s->_k;
        rest[j] = s->_rest;
        damp[j] = s->_damping;
        ty[j] = (int32_t)s->_type;
        om[j] = s->_omega;
        amp[j] = s->_amplitude;
        ph[j] = s->_phase;
    }
    check(titan_gb300_set_spring_params(handle, ns, nullptr, k.data(), rest.data(), damp.data(), ty.data(), om.data(),
                                        amp.data(), ph.data()),
          "setAll");
}

void Simulation::get(Container *c) {
    if (ENDED) throw std::runtime_error("The simulation has ended. Cannot get updates from the GPU after the end of the simulation.");
    if (!STARTED) {
        std::cerr << "sim.get() does nothing if called before the simulation has started." << std::endl;
        return;
    }
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    const int64_t n = (int64_t)c->masses.size();
    std::vector<int64_t> idx(n);
    for (int64_t i = 0; i < n; i++) idx[i] = c->masses[i]->index;
    std::vector<double> p(3 * n), v(3 * n), a(3 * n), t(n);
    check(titan_gb300_get_masses(handle, n, idx.data(), p.data(), v.data(), a.data(), t.data()), "get");
    for (int64_t i = 0; i < n; i++) {
        Mass *m = c->masses[i];
        m->pos = Vec(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
        m->vel = Vec(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        m->acc = Vec(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
        m->T = t[i];
    }
}

void Simulation::set(Container *c) {
    if (ENDED) throw std::runtime_error(kEnded);
    if (!STARTED) {
        std::cerr << "The simulation has not started. Get and set commands cannot be called before sim.start()" << std::endl;
        return;
    }
    std::lock_guard<std::mutex> lk(mu);
    syncTopology();
    const int64_t n = (int64_t)c->masses.size();
    std::vector<int64_t> idx(n);
    std::vector<double> p(3 * n), v(3 * n), m(n), e(3 * n), dr(n), t(n);
    std::vector<uint8_t> fx(n);
    for (int64_t i = 0; i < n; i++) {
        Mass *ms = c->masses[i];
        idx[i] = ms->index;
        for (int k = 0; k < 3; k++) {
            p[3 * i + k] = ms->pos[k];
            v[3 * i + k] = ms->vel[k];
            e[3 * i + k] = ms->extern_force[k];
        }
        m[i] = ms->m;
        dr[i] = ms->drag_coefficient;
        t[i] = ms->T;
        fx[i] = ms->fixed ? 1 : 0;
    }
    check(titan_gb300_set_mass_state(handle, n, idx.data(), p.data(), v.data(), m.data(), e.data(), fx.data(),
                                     dr.data(), t.data()),
          "set");
    const int64_t ns = (int64_t)c->springs.size();
    std::vector<int64_t> sidx(ns);
    std::vector<double> k(ns), rest(ns), damp(ns), om(ns), amp(ns), ph(ns);
    std::vector<int32_t> ty(ns);
    for (int64_t j = 0; j < ns; j++) {
        Spring *s = c->springs[j];
        sidx[j] = s->index;
        k[j] = s->_k;
        rest[j] = s->_rest;
        damp[j] = s->_damping;
        ty[j] = (int32_t)s->_type;
        om[j] = s->_omega;
        amp[j] = s->_amplitude;
        ph[j] = s->_phase;
    }
    if (ns > 0)
        check(titan_gb300_set_spring_params(handle, ns, sidx.data(), k.data(), rest.data(), damp.data(), ty.data(),
                                            om.data(), amp.data(), ph.data()),
              "set");
}

void Simulation::printPositions() {
    if (ENDED) throw std::runtime_error("The simulation has ended. You cannot view parameters of the simulation after it has been stopped.");
    if (STARTED) {
        std::cout << "\nDEVICE MASSES: " << std::endl;
        const int64_t n = (int64_t)masses.size();
        std::vector<double> p(3 * n);
        {
            std::lock_guard<std::mutex> lk(mu);
            check(titan_gb300_get_state(handle, p.data(), nullptr, nullptr, nullptr), "printPositions");
        }
        for (int64_t i = 0; i < n; i++) std::cout << i << ": " << Vec(p[3 * i], p[3 * i + 1], p[3 * i + 2]) << std::endl;
    } else {
        std::cout << "\nHOST MASSES: " << std::endl;
        int count = 0;
        for (Mass *m : masses) std::cout << count++ << ": " << m->pos << std::endl;
    }
    std::cout << std::endl;
}

Spring *Simulation::getSpringByIndex(int i) { return springs.at(i); }
Mass *Simulation::getMassByIndex(int i) { return masses.at(i); }
Container *Simulation::getContainerByIndex(int i) { return containers.at(i); }

}  // namespace titan
