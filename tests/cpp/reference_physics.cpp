// The reference's physics tests (test/physics/*.cpp, googletest) re-expressed
// without gtest against the drop-in header <Titan/sim.h>: same scenes, same
// control calls, same tolerances.  Run one test per process:
//     reference_physics <test_name>
// Exit status 0 = pass.
#include <Titan/sim.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <iostream>
#include <map>
#include <string>
#include <tuple>
#include <vector>

using titan::Vec;

static int failures = 0;

#define EXPECT_NEAR(a, b, tol)                                                                       \
    do {                                                                                             \
        double a_ = (a), b_ = (b), t_ = (tol);                                                       \
        if (!(std::fabs(a_ - b_) <= t_)) {                                                           \
            std::fprintf(stderr, "%s:%d: |%.9g - %.9g| > %.3g\n", __FILE__, __LINE__, a_, b_, t_);   \
            failures++;                                                                              \
        }                                                                                            \
    } while (0)
#define EXPECT_TRUE(c)                                                                 \
    do {                                                                               \
        if (!(c)) {                                                                    \
            std::fprintf(stderr, "%s:%d: expected %s\n", __FILE__, __LINE__, #c);      \
            failures++;                                                                \
        }                                                                              \
    } while (0)

// test/testutil/utils.h:12-30 (gravity PE with the hard-coded 9.8).  The
// penalty energy of masses below the z = 0 plane (20000 disp^2 / 2) is added:
// the reference's util omits it, which makes a sample taken inside a contact
// under-read by up to the whole kinetic energy.
static double energy(titan::Simulation &sim) {
    double pg = 0, ps = 0, ke = 0, pc = 0;
    sim.getAll();
    for (titan::Mass *m : sim.masses) {
        pg += 9.8 * (m->pos)[2] * (m->m);
        ke += 0.5 * (m->m) * std::pow((m->vel).norm(), 2);
        if (m->pos[2] < 0) pc += 0.5 * 20000.0 * m->pos[2] * m->pos[2];
    }
    for (titan::Spring *s : sim.springs) ps += s->_k * std::pow((s->_left->pos - s->_right->pos).norm() - s->_rest, 2) / 2;
    return ps + ke + pg + pc;
}

// test/physics/simple_unittest.cpp:15-34
static void simple_test() {
    titan::Simulation sim;
    sim.createMass(Vec(1, 0, 1));
    sim.setTimeStep(0.0001);
    sim.setGlobalAcceleration(Vec(0, 0, -9.8));
    sim.createPlane(Vec(0, 0, 1), 0);
    sim.start();
    double total = energy(sim), avg = total, alpha = 0.9;
    while (sim.time() < 5) {
        sim.wait(0.1);
        avg = (1 - alpha) * energy(sim) + alpha * avg;
        EXPECT_NEAR(avg, total, total * 0.01);
        sim.resume();
    }
    sim.stop();
}

// test/physics/energy_unittest.cpp:14-40
static void energy_test() {
    titan::Simulation sim;
    sim.createLattice(Vec(0, 0, 5), Vec(4, 4, 4), 20, 20, 20);
    sim.setAllSpringConstantValues(1000);
    sim.setTimeStep(0.0001);
    sim.setGlobalAcceleration(Vec(0, 0, -9.8));
    sim.defaultRestLengths();
    sim.createPlane(Vec(0, 0, 1), 0);
    sim.start();
    double total = energy(sim), avg = total, alpha = 0.7;
    while (sim.time() < 5) {
        sim.wait(0.1);
        avg = (1 - alpha) * energy(sim) + alpha * avg;
        EXPECT_NEAR(avg, total, total * 0.01);
        sim.resume();
    }
    sim.stop();
}

// test/physics/external_unittest.cpp:17-35
static void external_test() {
    titan::Simulation sim;
    titan::Mass *m1 = sim.createMass(Vec(1, 0, 1));
    sim.setTimeStep(0.0001);
    m1->setExternalForce(m1->m * Vec(0, 0, -9.8));
    sim.setGlobalAcceleration(Vec(0, 0, 0.0));
    sim.start();
    while (sim.time() < 5) {
        sim.wait(0.1);
        sim.getAll();
        EXPECT_NEAR(m1->pos[0], 1, 1e-6);
        EXPECT_NEAR(m1->pos[1], 0, 1e-6);
        EXPECT_NEAR(m1->pos[2], 1 + 0.5 * -9.8 * std::pow(sim.time(), 2), 0.1);
        sim.resume();
    }
    sim.stop();
}

// test/physics/external_unittest.cpp:38-56
static void external_acc_test() {
    titan::Simulation sim;
    titan::Mass *m1 = sim.createMass(Vec(1, 0, 1));
    sim.setTimeStep(0.0001);
    m1->setExternalForce(m1->m * Vec(0, 0, 0));
    sim.setGlobalAcceleration(Vec(0, 0, -9.8));
    sim.start();
    while (sim.time() < 1) {
        sim.wait(0.1);
        sim.getAll();
        EXPECT_NEAR(m1->pos[0], 1, 1e-6);
        EXPECT_NEAR(m1->pos[1], 0, 1e-6);
        EXPECT_NEAR(m1->pos[2], 1 + 0.5 * -9.8 * std::pow(sim.time(), 2), 0.1);
        sim.resume();
    }
    sim.stop();
}

// test/physics/multiagent_unittest.cpp:21-71 (smoke in the reference; here
// also: time reached, positions finite)
static void multiagent_test() {
    const double SIZE = 5.0, SPACE = 3.0;
    const int NUM_X = 10, NUM_Y = 10, DENSITY = 5;
    titan::Simulation sim;
    sim.setGlobalAcceleration(Vec(0, 0, -9.8));
    titan::Lattice *grid[NUM_Y][NUM_X];
    for (int i = 0; i < NUM_Y; i++)
        for (int j = 0; j < NUM_X; j++)
            grid[i][j] = sim.createLattice(Vec((SIZE + SPACE) * j + SIZE / 2, (SIZE + SPACE) * i + SIZE / 2, SIZE / 2),
                                           Vec(SIZE, SIZE, SIZE), DENSITY, DENSITY, DENSITY);
    std::vector<std::tuple<int, int>> right = {{100, 0}, {120, 20}, {104, 4}, {124, 24}};
    std::vector<std::tuple<int, int>> up = {{20, 0}, {120, 100}, {124, 104}, {24, 4}};
    for (int i = 0; i < NUM_Y - 1; i++)
        for (int j = 0; j < NUM_X - 1; j++) {
            for (auto pr : right) {
                titan::Spring *s = sim.createSpring(grid[i][j]->masses[std::get<0>(pr)], grid[i][j + 1]->masses[std::get<1>(pr)]);
                s->_k = 0.01;
                s->defaultLength();
            }
            for (auto pr : up) {
                titan::Spring *s = sim.createSpring(grid[i][j]->masses[std::get<0>(pr)], grid[i + 1][j]->masses[std::get<1>(pr)]);
                s->_k = 0.01;
                s->defaultLength();
            }
        }
    sim.defaultRestLengths();
    sim.start();
    sim.pause(1.0);
    sim.getAll();
    EXPECT_TRUE(sim.time() >= 1.0 && sim.time() < 1.0 + 2 * sim.getTimeStep());
    for (titan::Mass *m : sim.masses) EXPECT_TRUE(std::isfinite(m->pos[2]));
    sim.stop();
}

// test/physics/rotate_unittest.cpp:11-40 (smoke in the reference)
static void rotate_test() {
    titan::Simulation sim;
    titan::Lattice *l2 = sim.createLattice(Vec(0, 0, 10), Vec(5, 5, 5), 10, 10, 10);
    sim.setAllSpringConstantValues(1E5);
    l2->rotate(Vec(0, 0, 1), -0.78);
    sim.createPlane(Vec(0, 0, 1), 0, 10, 10);
    sim.setGlobalAcceleration(Vec(0, 0, -9.8));
    sim.start();
    while (true) {
        sim.pause(sim.time() + 1);
        sim.get(l2);
        l2->rotate(Vec(0, 0, 1), 0.5);
        sim.set(l2);
        if (sim.time() > 5.0) {
            for (titan::Mass *m : l2->masses) EXPECT_TRUE(std::isfinite(m->pos[2]));
            sim.stop();
            return;
        }
        sim.resume();
    }
}

// ---- extensions ----

// pause(t) stops at the first step whose accumulated time reaches t
// (src/sim.cu:1505); step(n) then advances exactly n steps.
static void breakpoint_and_step_test() {
    titan::Simulation sim;
    titan::Mass *m = sim.createMass(Vec(0, 0, 1));
    sim.setTimeStep(0.0001);
    sim.start();
    sim.pause(0.05);
    double t = 0;
    long n = 0;
    while (t < 0.05) {
        t += 0.0001;
        n++;
    }
    EXPECT_TRUE(sim.steps() == n);
    EXPECT_TRUE(sim.time() == t);
    sim.step(250);
    EXPECT_TRUE(sim.steps() == n + 250);
    sim.get(m);
    double v = 0, z = 1;
    for (long i = 0; i < n + 250; i++) {
        v = v + ((-9.81 * 0.1) / 0.1) * 0.0001;
        z = z + v * 0.0001;
    }
    EXPECT_NEAR(m->pos[2], z, 0.0);
    EXPECT_NEAR(m->T, sim.time(), 1e-15);
    sim.stop();
}

// Beam: the i == 0 face is fixed (src/object.cu:307-309) and never moves.
static void beam_fixed_face_test() {
    titan::Simulation sim;
    titan::Beam *b = sim.createBeam(Vec(0, 0, 2), Vec(2, 0.5, 0.5), 8, 3, 3);
    sim.start();
    sim.pause(0.2);
    sim.getAll();
    for (int i = 0; i < 9; i++) EXPECT_NEAR(b->masses[i]->pos[2], 2 + (i % 3) * 0.25 - 0.25, 1e-15);
    EXPECT_TRUE(b->masses.back()->pos[2] < 2.25);  // the free end sags
    sim.stop();
}

// createMass / createSpring while paused (src/sim.cu:223-341): existing
// masses keep their device state, new ones enter with their host state.
static void topology_edit_test() {
    titan::Simulation sim;
    titan::Mass *a = sim.createMass(Vec(0, 0, 5));
    sim.setGlobalAcceleration(Vec(0, 0, 0));
    a->vel = Vec(1, 0, 0);
    sim.start();
    sim.pause(0.1);
    titan::Mass *b = sim.createMass(Vec(0, 0, 10));
    titan::Spring *s = sim.createSpring(a, b);
    s->_k = 0;
    sim.resume();
    sim.pause(0.2);
    sim.getAll();
    EXPECT_NEAR(a->pos[0], sim.steps() * 0.0001, 1e-12);
    EXPECT_NEAR(b->pos[2], 10, 0.0);
    EXPECT_TRUE(sim.masses.size() == 2 && sim.springs.size() == 1);
    sim.stop();
}

// deleteSpring / deleteMass / deleteContainer while paused (src/sim.cu:
// 351-410, 510-563): a 6^3 lattice and a 4^3 lattice fall onto a
// frictional plane; after the first pause four springs of the first lattice,
// one of its masses (whose springs are then skipped, src/sim.cu:1052) and the
// whole second lattice are deleted, and the run resumes.  The remaining
// masses' state is written to the file named on the command line
// (int64 steps before and after the deletion, int64 mass count, then pos
// and vel of each mass in sim.masses order, doubles) for the oracle to check.
static const char *g_dump_path = nullptr;
static void delete_after_start_test() {
    titan::Simulation sim;
    titan::Lattice *a = sim.createLattice(Vec(0, 0, 0.6), Vec(1, 1, 1), 6, 6, 6);
    titan::Lattice *b = sim.createLattice(Vec(3, 0, 0.6), Vec(1, 1, 1), 4, 4, 4);
    sim.createPlane(Vec(0, 0, 1), 0, 0.5, 0.5);
    sim.start();
    sim.pause(0.05);
    const int64_t n1 = sim.steps();
    for (int j : {0, 7, 100, 333}) sim.deleteSpring(a->springs[j]);
    sim.deleteMass(a->masses[40]);
    sim.deleteContainer(b);
    EXPECT_TRUE(sim.masses.size() == 215);
    sim.resume();
    sim.pause(0.2);
    const int64_t n2 = sim.steps() - n1;
    sim.getAll();
    EXPECT_TRUE(g_dump_path != nullptr);
    if (!g_dump_path) return;
    FILE *f = std::fopen(g_dump_path, "wb");
    EXPECT_TRUE(f != nullptr);
    if (!f) return;
    const int64_t head[3] = {n1, n2, (int64_t)sim.masses.size()};
    std::fwrite(head, 8, 3, f);
    for (titan::Mass *m : sim.masses) {
        const double rec[6] = {m->pos[0], m->pos[1], m->pos[2], m->vel[0], m->vel[1], m->vel[2]};
        std::fwrite(rec, 8, 6, f);
    }
    std::fclose(f);
    sim.stop();
}

// importFromSTL (src/sim.cu:1855-1921): a binary STL of an L-shaped solid
// (two closed boxes, [0,2]x[0,1]x[0,1] and [0,1]x[1,2]x[0,1]) written here;
// the bounding box [0,2]x[0,2]x[0,1] gets a 10^3 lattice, and the masses in
// the missing quadrant are dropped with their springs.
static void stl_import_test() {
    // a per-run file name, so that concurrent runs do not share the fixture
    char path[] = "/tmp/titan_gb300_stl_XXXXXX";
    {
        const int fd = mkstemp(path);
        EXPECT_TRUE(fd >= 0);
        if (fd < 0) return;
        FILE *f = fdopen(fd, "wb");
        EXPECT_TRUE(f != nullptr);
        if (!f) return;
        char header[80] = {0};
        std::fwrite(header, 1, 80, f);
        const uint32_t n = 24;
        std::fwrite(&n, 4, 1, f);
        const float boxes[2][2][3] = {{{0, 0, 0}, {2, 1, 1}}, {{0, 1, 0}, {1, 2, 1}}};
        const int q[6][4] = {{0, 2, 3, 1}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 6, 7, 3}, {0, 4, 6, 2}, {1, 3, 7, 5}};
        for (const auto &b : boxes) {
            float c[8][3];
            for (int i = 0; i < 8; i++)
                for (int d = 0; d < 3; d++) c[i][d] = ((i >> d) & 1) ? b[1][d] : b[0][d];
            for (const auto &quad : q)
                for (int h = 0; h < 2; h++) {
                    const int v[3] = {quad[0], quad[h + 1], quad[h + 2]};
                    float rec[12] = {0, 0, 0};
                    for (int k = 0; k < 3; k++)
                        for (int d = 0; d < 3; d++) rec[3 + 3 * k + d] = c[v[k]][d];
                    const uint16_t attr = 0;
                    std::fwrite(rec, 4, 12, f);
                    std::fwrite(&attr, 2, 1, f);
                }
        }
        std::fclose(f);
    }
    titan::Simulation sim;
    // density 2.1: num_pts = (int) cbrt(2.1 * (10 / 2)^3 * 2 * 2 * 1) = 10
    titan::Container *c = sim.importFromSTL(path, 2.1, 5);
    std::remove(path);
    // lattice point (px, py, pz) maps to (1 + 0.2 px, 1 + 0.2 py, 0.2 (pz - 5) + 0.5)
    int kept_expected = 0;
    for (int i = 0; i < 10; i++)
        for (int j = 0; j < 10; j++) {
            const double x = 1 + 0.2 * (-4.9995 + i * 9.999 / 9), y = 1 + 0.2 * (-4.9995 + j * 9.999 / 9);
            if (y < 1 || x < 1) kept_expected += 10;
        }
    EXPECT_TRUE((int)c->masses.size() == kept_expected);
    for (titan::Mass *m : c->masses) {
        const double x = 1.0 + 0.2 * m->pos[0], y = 1.0 + 0.2 * m->pos[1];
        EXPECT_TRUE(y < 1 || x < 1);
    }
    for (titan::Spring *sp : c->springs) {
        bool l = false, r = false;
        for (titan::Mass *m : c->masses) {
            l = l || m == sp->_left;
            r = r || m == sp->_right;
        }
        EXPECT_TRUE(l && r);
    }
    EXPECT_TRUE(sim.masses.size() == c->masses.size() && sim.springs.size() == c->springs.size());
    sim.start();
    sim.pause(0.01);
    sim.getAll();
    EXPECT_TRUE(std::isfinite(c->masses[0]->pos[2]) && c->masses[0]->pos[2] < 10.0);
    sim.stop();
}

// Throws std::runtime_error whose message contains `what`.
template <class F>
static bool throws_with(F &&f, const char *what) {
    try {
        f();
    } catch (const std::runtime_error &e) {
        return std::strstr(e.what(), what) != nullptr;
    }
    return false;
}

// The reference's misuse conventions before start() (src/sim.cu:798-806,
// 1348-1356, 1484-1495, 590, 944): start() without masses, a non-positive
// time step and resume() before start() throw with the reference's messages;
// get() before start() prints and leaves the host objects alone.  Host-only
// bulk edits (src/sim.cu:780-796) apply before start.  No device is touched.
static void errors_test() {
    titan::Simulation sim;
    EXPECT_TRUE(throws_with([&] { sim.start(); }, "No masses have been added"));
    EXPECT_TRUE(throws_with([&] { sim.setTimeStep(0.0); }, "Cannot set time step to negative or zero value."));
    EXPECT_TRUE(throws_with([&] { sim.setTimeStep(-1e-4); }, "Cannot set time step to negative or zero value."));
    EXPECT_NEAR(sim.getTimeStep(), 0.0001, 0);
    sim.setTimeStep(2e-4);
    EXPECT_NEAR(sim.getTimeStep(), 2e-4, 0);
    EXPECT_TRUE(throws_with([&] { sim.resume(); }, "You cannot resume a simulation before calling sim.start()"));
    EXPECT_TRUE(throws_with([&] { sim.setPrecision(3); }, "precision must be"));

    titan::Mass *a = sim.createMass(Vec(0, 0, 1));
    titan::Mass *b = sim.createMass(Vec(0, 0, 2));
    titan::Spring *s = sim.createSpring(a, b);
    EXPECT_TRUE(sim.masses.size() == 2 && sim.springs.size() == 1);
    EXPECT_NEAR(s->_rest, 1.0, 1e-15);
    sim.setAllMassValues(0.5);  // adds, as the reference does
    EXPECT_NEAR(a->m, 0.6, 1e-15);
    sim.setAllSpringConstantValues(123.0);
    EXPECT_NEAR(s->_k, 123.0, 0);
    b->pos = Vec(0, 0, 4);
    sim.defaultRestLengths();
    EXPECT_NEAR(s->_rest, 3.0, 1e-15);

    a->pos = Vec(7, 8, 9);
    sim.get(a);  // not started: prints, changes nothing
    EXPECT_NEAR(a->pos[0], 7, 0);
    titan::Container *c = sim.createContainer();
    c->add(a);
    sim.get(c);
    EXPECT_NEAR(a->pos[2], 9, 0);
    EXPECT_TRUE(throws_with([&] { sim.resume(); }, "You cannot resume"));
    sim.setBreakpoint(1.0);  // allowed before start
}

int main(int argc, char **argv) {
    std::map<std::string, void (*)()> tests = {
        {"errors_test", errors_test},
        {"simple_test", simple_test},         {"energy_test", energy_test},
        {"external_test", external_test},     {"external_acc_test", external_acc_test},
        {"multiagent_test", multiagent_test}, {"rotate_test", rotate_test},
        {"breakpoint_and_step_test", breakpoint_and_step_test},
        {"beam_fixed_face_test", beam_fixed_face_test},
        {"topology_edit_test", topology_edit_test},
        {"stl_import_test", stl_import_test},
        {"delete_after_start_test", delete_after_start_test},
    };
    if (argc < 2 || !tests.count(argv[1])) {
        for (auto &kv : tests) std::printf("%s\n", kv.first.c_str());
        return argc < 2 ? 0 : 2;
    }
    if (argc > 2) g_dump_path = argv[2];
    try {
        tests[argv[1]]();
    } catch (const std::exception &e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 3;
    }
    std::printf("%s: %s\n", argv[1], failures ? "FAILED" : "ok");
    return failures ? 1 : 0;
}
