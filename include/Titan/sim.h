// Titan/sim.h -- titan::Simulation, the drop-in for Titan's user API
// (include/Titan/sim.h:37-220 in the reference), implemented over the C ABI of
// titan_gb300.h.  Same member names, signatures, defaults and error
// conventions (std::runtime_error on misuse); graphics members are absent.
//
// Run model: start() uploads the scene and starts a request loop on a host
// thread that advances the simulation in CUDA-graph chunks until the next
// breakpoint (simulated time, as src/sim.cu:1505 checks it); pause/wait/
// resume/stop control it as in the reference.  get/set/getAll/setAll move
// state between the host objects and the device between chunks.
#ifndef TITAN_GB300_SIM_H
#define TITAN_GB300_SIM_H

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "mass.h"
#include "object.h"
#include "spring.h"
#include "vec.h"

struct titan_gb300_sim;

namespace titan {

class Simulation {
public:
    // Create
    Mass *createMass();
    Mass *createMass(const Vec &pos);
    Spring *createSpring();
    Spring *createSpring(Mass *m1, Mass *m2);

    // Delete
    void deleteMass(Mass *m);
    void deleteSpring(Spring *s);

    void get(Mass *m);
    void get(Spring *s);
    void get(Container *c);
    void set(Mass *m);
    void set(Spring *s);
    void set(Container *c);
    void getAll();
    void setAll();

    // Global constraints
    void createPlane(const Vec &abc, double d);
    void createPlane(const Vec &abc, double d, double FRICTION_K, double FRICTION_S);
    void createBall(const Vec &center, double r);
    void clearConstraints();

    // Containers
    Container *createContainer();
    void deleteContainer(Container *c);
    Cube *createCube(const Vec &center, double side_length);
    Lattice *createLattice(const Vec &center, const Vec &dims, int nx = 10, int ny = 10, int nz = 10);
    Beam *createBeam(const Vec &center, const Vec &dims, int nx = 10, int ny = 10, int nz = 10);
    // Binary STL import (src/sim.cu:1855-1921): a num_pts^3 lattice over the
    // mesh's bounding box, keeping the masses whose point the mesh contains
    // (ray-parity point-in-mesh test on the GPU, seeded rays) and the springs
    // between them.  Throws std::runtime_error when the file cannot be read
    // or is not a binary STL.
    Container *importFromSTL(const std::string &path, double density = 10.0, int num_rays = 5);

    // Bulk modifications, host objects only
    void setAllSpringConstantValues(double k);
    void setAllMassValues(double m);  // adds m, as the reference does (src/sim.cu:788-795)
    void setTimeStep(double delta_t);
    double getTimeStep();
    void setGlobalAcceleration(const Vec &global_acc);
    void defaultRestLengths();

    // Control
    void start();
    void stop();
    void stop(double time);
    void pause(double t);
    void resume();
    void reset();
    void setBreakpoint(double time);
    void wait(double t);
    void waitUntil(double t);
    void waitForEvent();
    double time();
    bool running();

    void printPositions();

    Simulation();
    ~Simulation();

    Spring *getSpringByIndex(int i);
    Mass *getMassByIndex(int i);
    Container *getContainerByIndex(int i);

    std::vector<Mass *> masses;
    std::vector<Spring *> springs;
    std::vector<Container *> containers;

    // ---- extensions (no counterpart in the reference) ----
    // Run exactly n steps now (simulation started and paused); returns when done.
    void step(long n);
    // Arithmetic of the step: 0 FP64 (default), 1 FP32, 2 FP32 compensated;
    // set before start().  The environment variable TITAN_GB300_PRECISION
    // gives the default.
    void setPrecision(int precision);
    int precision() const { return precision_; }
    long steps();
    // Device-side FP64 diagnostics: energy[4] = spring PE, kinetic, gravity PE
    // (g_mag z m), total; momentum[6] = linear, angular.
    void diagnostics(double g_mag, double energy[4], double momentum[6]);

private:
    Mass *createMass(Mass *m);
    Spring *createSpring(Spring *s);
    void buildDevice(bool keep_device_state);
    void loop();
    void check(int rc, const char *what);
    void requireStarted(const char *what);
    void syncTopology();

    double dt;
    std::atomic<double> T{0.0};
    std::atomic<bool> RUNNING{false}, STARTED{false}, ENDED{false}, FREED{false}, GPU_DONE{false};
    Vec _global_acc;
    struct Plane {
        Vec n;
        double d, fk, fs;
    };
    struct Ball {
        Vec c;
        double r;
    };
    std::vector<Plane> planes;
    std::vector<Ball> balls;
    std::set<double> bpts;
    std::vector<Mass *> graveyard;
    std::vector<Spring *> spring_graveyard;
    titan_gb300_sim *handle = nullptr;
    long steps_base = 0;  // steps run by handles replaced in topology rebuilds
    int precision_ = 0;
    bool dirty = false;  // topology changed since the device scene was built
    std::vector<Mass *> built_masses;
    std::vector<Spring *> built_springs;
    std::vector<std::pair<Mass *, Mass *>> built_ends;
    std::mutex mu;
    std::condition_variable cv;
    std::thread gpu_thread;
};

}  // namespace titan

#endif
