/*
 * titan_gb300.h -- C ABI of the GB300 mass-spring step engine.
 *
 * This is the drop-in boundary for the hot path of Titan's titan::Simulation
 * (include/Titan/sim.h:37-220 in the reference).  The reference has no C ABI
 * of its own: its boundary is the C++ class.  Each entry point below names
 * the reference member function whose device-side work it replaces; the C++
 * shim in include/Titan/sim.h (this repository) maps those member functions
 * onto these calls one to one.
 *
 * Conventions
 *   - Every call returns an int status (TITAN_GB300_OK == 0); no C++
 *     exception crosses this boundary.  titan_gb300_last_error() gives the
 *     message of the last failed call on that handle.
 *   - Vectors are xyz-interleaved doubles: mass i's position is pos[3i..3i+2].
 *   - Host buffers belong to the caller and are not retained after a call.
 *   - Work is queued on the handle's own CUDA stream; calls that return data
 *     to the host synchronise that stream first.
 *   - Masses and springs are addressed by their index in the arrays the
 *     caller uploaded (creation order in titan::Simulation).  Internally the
 *     engine renumbers masses into spatial tiles; that order never leaks out.
 */
#ifndef TITAN_GB300_H
#define TITAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TITAN_GB300_OK 0
#define TITAN_GB300_EINVAL 1      /* bad argument or call order          */
#define TITAN_GB300_ECUDA 2       /* CUDA runtime error                   */
#define TITAN_GB300_ENOMEM 3      /* device or host allocation failed     */
#define TITAN_GB300_ELIMIT 4      /* scene exceeds a documented limit     */
#define TITAN_GB300_ESTATE 5      /* simulation ended / not started       */
#define TITAN_GB300_ETIMEOUT 6    /* a bounded wait gave up               */
#define TITAN_GB300_EBUDGET 7     /* serving admission over HBM budget    */
#define TITAN_GB300_EBUSY 8       /* poll: queued steps still running     */

/* Arithmetic of the step.  FP64 is the drop-in form (reference kernels are
 * FP64).  FP32 runs positions/velocities in single precision.  FP32C runs the
 * force arithmetic in FP32 and keeps positions and velocities as compensated
 * (hi + lo) float pairs. */
#define TITAN_GB300_FP64 0
#define TITAN_GB300_FP32 1
#define TITAN_GB300_FP32C 2

/* Spring types: include/Titan/spring.h:17. */
#define TITAN_GB300_PASSIVE_SOFT 0
#define TITAN_GB300_PASSIVE_STIFF 1
#define TITAN_GB300_ACTIVE_CONTRACT_THEN_EXPAND 2
#define TITAN_GB300_ACTIVE_EXPAND_THEN_CONTRACT 3

/* Local constraint types: include/Titan/object.h:223-225 (CONSTRAINT_TYPE). */
#define TITAN_GB300_CONSTRAINT_PLANE 0
#define TITAN_GB300_CONTACT_PLANE 1
#define TITAN_GB300_BALL 2
#define TITAN_GB300_DIRECTION 3

typedef struct titan_gb300_sim titan_gb300_sim;

/* ---- lifecycle --------------------------------------------------------- */

/* Replaces Simulation::Simulation() (src/sim.cu:77-100): dt = 1e-4,
 * g = (0, 0, -9.81).  device: CUDA ordinal; precision: TITAN_GB300_FP*. */
int titan_gb300_create(titan_gb300_sim **out, int device, int precision);

/* Replaces Simulation::~Simulation() / freeGPU() (src/sim.cu:131-221). */
void titan_gb300_destroy(titan_gb300_sim *sim);

/* Message of the last failed call on sim (never NULL). */
const char *titan_gb300_last_error(const titan_gb300_sim *sim);

/* ---- scene, host side (before start, or while paused) ------------------ */

/* Replaces createMass (src/sim.cu:223-289) for a whole array of masses, plus
 * Mass::setExternalForce / fix / setDrag (include/Titan/mass.h:27-38).
 * vel, ext_force, fixed, drag may be NULL (zero / not fixed / no drag).  The
 * drag coefficient is truncated to int as the reference's device struct does
 * (include/Titan/object.h:213). */
int titan_gb300_set_masses(titan_gb300_sim *sim, int64_t n, const double *pos,
                           const double *vel, const double *m, const double *ext_force,
                           const uint8_t *fixed, const double *drag);

/* Replaces createSpring (src/sim.cu:291-341) for a whole array, with the
 * actuation fields _type/_omega/_damping (include/Titan/spring.h:49-55).
 * left/right = -1 means no mass attached (the reference then skips the spring,
 * src/sim.cu:1052).  type, omega may be NULL (passive).  amp and phase extend
 * the reference's fixed 0.2 sin(omega t) actuation: NULL means amp = 0.2,
 * phase = 0, which reproduces the reference exactly. */
int titan_gb300_set_springs(titan_gb300_sim *sim, int64_t n, const int32_t *left,
                            const int32_t *right, const double *k, const double *rest,
                            const double *damping, const int32_t *type, const double *omega,
                            const double *amp, const double *phase);

/* Replaces Mass::addConstraint (src/mass.cu:78-101) for all masses at once:
 * records of mass i are mass_ptr[i] .. mass_ptr[i+1]-1 (mass_ptr has n+1
 * entries), vec/num as given to addConstraint (normalised here as the
 * reference constructors do).  Records are applied in the reference's order:
 * contact planes, balls, constraint planes, directions (src/sim.cu:1117-1131). */
int titan_gb300_set_local_constraints(titan_gb300_sim *sim, const int64_t *mass_ptr,
                                      const int32_t *type, const double *vec, const double *num);

/* Replaces createPlane (src/sim.cu:1998-2023); normal is normalised. */
int titan_gb300_add_plane(titan_gb300_sim *sim, const double normal[3], double offset,
                          double friction_k, double friction_s);

/* Replaces createBall (src/sim.cu:2025-2035). */
int titan_gb300_add_ball(titan_gb300_sim *sim, const double center[3], double radius);

/* Replaces clearConstraints (src/sim.cu:2037-2040): removes global planes and balls. */
int titan_gb300_clear_constraints(titan_gb300_sim *sim);

/* Integrator of the mass update: 0 = symplectic Euler (the reference's
 * default build, src/sim.cu:1161-1166), 1 = VERLET (its -DVERLET build,
 * :1155-1159; the acceleration is state and starts at 0), 2 = RK2 (its -DRK2
 * build, :1141-1154 and :1572-1583: spring forces at T and at T + dt/2, time
 * advanced by dt/2 twice per step).  The reference chooses at compile time;
 * here it may change between steps.  Resident bins run Euler only. */
#define TITAN_GB300_EULER 0
#define TITAN_GB300_VERLET 1
#define TITAN_GB300_RK2 2
int titan_gb300_set_integrator(titan_gb300_sim *sim, int kind);

/* Replaces setTimeStep (src/sim.cu:797-807); dt <= 0 is EINVAL. */
int titan_gb300_set_time_step(titan_gb300_sim *sim, double dt);
double titan_gb300_get_time_step(const titan_gb300_sim *sim);

/* Replaces setGlobalAcceleration (src/sim.cu:2081-2087). */
int titan_gb300_set_global_acc(titan_gb300_sim *sim, const double g[3]);

/* Groups masses into independent bodies: body b owns masses
 * mass_ptr[b] .. mass_ptr[b+1]-1 (creation order, contiguous).  Tiles never
 * straddle two bodies.  Optional; without it the scene is one body. */
int titan_gb300_set_bodies(titan_gb300_sim *sim, int64_t nbodies, const int64_t *mass_ptr);

/* Per-body ground plane (a contact plane with friction that acts only on the
 * masses of that body).  normal is normalised. */
int titan_gb300_set_body_plane(titan_gb300_sim *sim, int64_t body, const double normal[3],
                               double offset, double friction_k, double friction_s);

/* ---- device side -------------------------------------------------------- */

/* Replaces start() (src/sim.cu:1349-1390) minus the thread spawn: builds the
 * tile plan (spatial renumbering, spring slabs, per-mass incidence), uploads
 * the structure-of-arrays state and resets time to 0.  tile_masses = 0 picks
 * the tuned default: near-cubic tiles of up to 208 masses for the FP32 forms'
 * warp-specialised kernel (192 where two of them would not fit one SM's
 * shared memory), 256 for the per-tile forms and in FP64; smaller for small
 * scenes, so that their tiles cover the SMs (about 4 tiles per SM, at least
 * 64 masses, in the FP32 forms; about 1.6, at least 32, in FP64); in the
 * FP32 forms a body that fits the large tile stays one tile. */
int titan_gb300_start(titan_gb300_sim *sim, int tile_masses);

/* Takes src's tile plan for this handle's next start() instead of building
 * one (no reference counterpart: for serving many scenes of one topology).
 * src must have been planned (plan_host) or started; both handles must have
 * the same precision, kernel form, masses, springs (ends), fixed masses,
 * actuated springs and bodies -- positions, parameters and constraints may
 * differ.  The plan is used when start()'s requested tile size equals the
 * one src was planned with (0 for both: the default).  Results
 * do not depend on which plan a scene runs with. */
int titan_gb300_adopt_plan(titan_gb300_sim *sim, const titan_gb300_sim *src);

/* Launch shape of the step kernel: threads per CTA, a multiple of 32 in
 * [64, 512], or 0 to derive it from the tile size.  Set before start(); the
 * tile size itself is start()'s argument.  Used by the autotuner. */
int titan_gb300_set_launch(titan_gb300_sim *sim, int threads_per_cta);

/* Register cap of the per-tile step kernel in the FP32 forms: 0 or 1 = none
 * (up to 128 registers per thread), 3 or 4 = compile-time launch bounds for
 * 3 or 4 resident CTAs per SM of at most 256 threads (85 / 64 registers).
 * More resident warps hide more memory latency; fewer registers may spill.
 * FP64 ignores it.  Set before start(); start() fails with EINVAL when the
 * CTA is larger than 256 threads.  Used by the autotuner. */
int titan_gb300_set_occupancy(titan_gb300_sim *sim, int min_ctas_per_sm);

/* Step kernel form (extension; the reference has one pair of kernels):
 * 0 = automatic: the warp-specialised kernel in FP32 and FP32C (measured
 * fastest on GB300), the per-tile kernel in FP64, and resident tiles for
 * halo-free tiles (set_resident); 1 = per-tile kernel (one CTA per tile);
 * 3 = per-tile kernel whose slab records and tile states arrive by bulk
 * copy (TMA) and halo by cp.async, all issued before one wait; 4 =
 * warp-specialised persistent kernel (a producer warp streams tiles into a
 * shared-memory ring, two consumer groups compute; fails at start() when two
 * tiles do not fit); 6 = pull kernel, FP32 and FP32C only (every mass sums
 * its own springs' forces from streamed spring columns against tile states
 * a producer warp stages; fails at start() in FP64 or with a mass above the
 * heavy threshold).  All forms give bit-identical results.  Set before
 * start(). */
int titan_gb300_set_kernel(titan_gb300_sim *sim, int variant);

/* After start(): out[0] kernel form of the per-step launches (1 to 4; 5
 * when resident tiles carry the whole scene and no per-step kernel runs),
 * out[1] CTAs per launch, out[2] threads per CTA, out[3] dynamic shared
 * memory per CTA (bytes) -- of the resident-tile launch for form 5. */
int titan_gb300_kernel_info(const titan_gb300_sim *sim, int64_t out[4]);

/* Batched bodies (no reference counterpart: the reference runs one scene
 * per process, src/sim.cu:1503-1617).  With resident bins on, every body
 * (set_bodies) that fits one CTA -- no spring to another body, every free
 * mass of degree <= 254, 2 state records per mass in shared memory -- is
 * packed with others into a bin of at most bin_masses masses, and one
 * persistent launch per step() call runs all nsteps steps of every bin with
 * the state held in shared memory; the remaining bodies take the per-step
 * kernels.  Results are bit-identical to the per-step kernels.
 *   mode -1 (default): automatic -- resident tiles (mode 2) for the
 *   scene's halo-free tiles when the kernel form is automatic (set_kernel
 *   0) and the integrator is symplectic Euler (measured on GB300: 2.5x
 *   faster than the per-step kernels on one 125-mass body, 2x on thousands
 *   of small bodies, 5 % on a batch whose small bodies alone are
 *   halo-free), else off; 0 off; 1 bins of
 *   whole bodies, one thread per mass (bin_masses: bin capacity, rounded
 *   up to a multiple of 32; 0: the largest fitting body when at most 152
 *   bodies fit, else max(1024, largest fitting body); bodies above it are
 *   not resident); 2 resident tiles: every tile with no halo (all springs
 *   of its masses inside it) is stepped by one CTA for all steps of a call
 *   with the per-step kernels' two phases in shared memory, its slab,
 *   actuation and incidence records staged there too when they fit and
 *   every such tile still gets a CTA at once (bin_masses unused; the tile
 *   size is start()'s).  threads_per_cta 0: derived from the bin or tile
 *   size; else a multiple of 32 in [64, 512].  Symplectic Euler only: the
 *   other integrators run every tile on the per-step kernels.
 * Set before start(). */
int titan_gb300_set_resident(titan_gb300_sim *sim, int mode, int bin_masses, int threads_per_cta);

/* After start(): out[0] the resident form in use (0 none, 1 bins, 2
 * tiles), out[1] bins or resident tiles, out[2] resident bodies, out[3]
 * resident masses, out[4] bin capacity or largest resident tile (masses),
 * out[5] threads per CTA, out[6] CTAs per launch, out[7] dynamic shared
 * memory per CTA (bytes). */
int titan_gb300_resident_info(const titan_gb300_sim *sim, int64_t out[8]);

/* One iteration of the reference's execute() loop body (src/sim.cu:1569-1590)
 * nsteps times: spring forces + mass update fused into one kernel per step,
 * replayed from cached CUDA graphs.  Asynchronous. */
int titan_gb300_step(titan_gb300_sim *sim, int64_t nsteps);

/* Extension (no counterpart in the reference, whose execute() loop launches
 * kernels directly): builds and caches the CUDA graphs that step(nsteps)
 * would replay from the current step parity, without launching anything, so
 * that a later step(nsteps) spends no host time on graph capture.  Graphs
 * are dropped when the scene is rebuilt (integrator switch, topology change). */
int titan_gb300_prepare_steps(titan_gb300_sim *sim, int64_t nsteps);

/* Wait for queued work; replaces the cudaDeviceSynchronize at src/sim.cu:1570.
 * TITAN_GB300_ETIMEOUT from here, poll or wait (not wait's own time limit)
 * means a step kernel's bounded wait for its shared-memory copies gave up:
 * the kernel stopped early, so the scene's state is undefined and the
 * handle must be destroyed. */
int titan_gb300_synchronize(titan_gb300_sim *sim);

/* step() is the asynchronous rollout launch.  poll(): TITAN_GB300_OK when
 * every queued step has finished, TITAN_GB300_EBUSY while some still run (a
 * non-blocking replacement for the reference's running()/waitForEvent()
 * spin, src/sim.cu:1628-1657).  wait(): blocks up to timeout_ms, then
 * TITAN_GB300_ETIMEOUT with the work still queued. */
int titan_gb300_poll(titan_gb300_sim *sim);
int titan_gb300_wait(titan_gb300_sim *sim, double timeout_ms);

/* Headless replacements of the reference's OpenGL export kernels.
 * export_vertices: the positions of all masses in creation order as 3n
 * floats, (float) of the position (updateVertices, src/sim.cu:1717-1725).
 * export_indices: 2 * ns uint32 -- each spring's left and right mass index,
 * (0, 0) for a spring without both masses (updateIndices,
 * src/sim.cu:1727-1750).  out_on_device != 0: out is device memory and the
 * vertex copy is queued on the handle's stream (no host synchronisation);
 * else out is host memory and the call returns when it is filled. */
int titan_gb300_export_vertices(titan_gb300_sim *sim, float *out, int out_on_device);
int titan_gb300_export_indices(titan_gb300_sim *sim, uint32_t *out, int out_on_device);

/* Replaces time() (src/sim.cu:1082): host-accumulated T (T += dt per step). */
double titan_gb300_time(const titan_gb300_sim *sim);

/* Device memory held by the handle (bytes), for admission control. */
int64_t titan_gb300_device_bytes(const titan_gb300_sim *sim);

/* Page-locked host memory (cudaMallocHost) for state buffers: get_state,
 * get_masses and set_mass_state move a page-locked caller buffer by DMA
 * directly, any other buffer through the handle's own page-locked staging
 * copy.  host_alloc returns NULL on failure; host_free accepts NULL.
 * Extension (the reference moves state through its own pinned-less
 * cudaMemcpy, src/sim.cu:588-764). */
void *titan_gb300_host_alloc(size_t bytes);
void titan_gb300_host_free(void *p);

/* Number of steps run since start(). */
int64_t titan_gb300_steps(const titan_gb300_sim *sim);

/* Sets T (the time the next step's actuation sees).  The reference sets T = 0
 * in start() (src/sim.cu:1369); this lets a host rebuild a scene mid-run
 * (topology edited while paused) and continue at the same time. */
int titan_gb300_set_time(titan_gb300_sim *sim, double T);

/* Replaces getAll() / massFromArray (src/sim.cu:642-653, 983-1005): copies
 * pos, vel, acc (3n each) and per-mass local time T (n) back in creation
 * order.  Any pointer may be NULL. */
int titan_gb300_get_state(titan_gb300_sim *sim, double *pos, double *vel, double *acc,
                          double *T);

/* get(Mass*) (src/sim.cu:588-601) for a list of masses. */
int titan_gb300_get_masses(titan_gb300_sim *sim, int64_t count, const int64_t *idx,
                           double *pos, double *vel, double *acc, double *T);

/* Replaces setAll() / set(Mass*) / set(Container*) (src/sim.cu:603-615,
 * 655-766) for masses: overwrites pos, vel, m, extern force, fixed, drag and
 * local time of the listed masses (idx == NULL: all n, in order).  Any data
 * pointer may be NULL to leave that field unchanged.  Forces restart at 0. */
int titan_gb300_set_mass_state(titan_gb300_sim *sim, int64_t count, const int64_t *idx,
                               const double *pos, const double *vel, const double *m,
                               const double *ext_force, const uint8_t *fixed,
                               const double *drag, const double *T);

/* Replaces set(Spring*) / the spring half of setAll() (src/sim.cu:632-640,
 * 746-764): new k, rest, damping, type, omega (and the amp/phase extension)
 * for the listed springs (idx == NULL: all).  Endpoints cannot change here.
 * NULL leaves a field unchanged. */
int titan_gb300_set_spring_params(titan_gb300_sim *sim, int64_t count, const int64_t *idx,
                                  const double *k, const double *rest, const double *damping,
                                  const int32_t *type, const double *omega, const double *amp,
                                  const double *phase);

/* FP64 diagnostics on the device, following test/testutil/utils.h:12-43:
 * energy[4] = {spring PE, kinetic, gravity PE (g_mag * z * m), total};
 * momentum[6] = {linear xyz, angular xyz} with angular = sum cross(m v, x).
 * Either output may be NULL.  Deterministic (fixed-order two-pass reduction). */
int titan_gb300_diagnostics(titan_gb300_sim *sim, double g_mag, double energy[4],
                            double momentum[6]);

/* The same FP64 energy and momentum as titan_gb300_diagnostics, for callers
 * that must not allocate device memory when they ask (memory reserved once at
 * start-up, a host framework whose caching allocator owns the device, work
 * issued while a stream is being captured).  No counterpart in the reference.
 * It allocates nothing: inputs and the output are the caller's device
 * buffers -- pos, vel (3n doubles, xyz-interleaved), m (n), left/right (ns
 * int32, -1 = skipped), k, rest (ns) -- and out receives 9 doubles (spring
 * PE, kinetic, gravity PE = g_mag z m, linear momentum xyz, angular momentum
 * xyz), queued on stream (a cudaStream_t, NULL = default stream).  Scratch
 * is a 288 KiB array compiled into the library, held on every GPU that loads
 * it until the process exits.  n and ns may be at most 4096 * 256 * 64
 * (67,108,864); larger sizes return TITAN_GB300_ELIMIT without launching.
 * The first call on a device looks the array's address up
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * Calls share the array: two calls that overlap on the GPU race and must be
 * ordered by the caller. */
int titan_gb300_diagnostics_noalloc(const double *pos, const double *vel, const double *m, int64_t n,
                                    const int32_t *left, const int32_t *right, const double *k,
                                    const double *rest, int64_t ns, double g_mag, double *out,
                                    void *stream);

/* ---- device-resident request server ---------------------------------------
 * Extension with no counterpart in the reference, which runs one scene per
 * process on a host thread that launches two kernels per step
 * (src/sim.cu:1389-1428, 1503-1617).  A server is one persistent kernel
 * (cooperative launch, one CTA per SM) that steps many started scenes at
 * once: each submitted scene takes a slot, is admitted at the next step
 * boundary and stepped nsteps times with the per-tile kernel's arithmetic
 * (bit-identical to the scene's own step(), whatever else is running), and
 * its slot is freed when its steps are done.  Submissions go through a ring
 * in page-locked host memory that the kernel reads between steps; finished
 * requests are reported in page-locked memory the host polls.  The kernel
 * leaves after a second without work and is launched again by the next
 * submit or poll; every wait in it is bounded.
 *   create: max_slots scenes at once (1 to 16384); tile_smem_bytes of
 *     shared memory for one tile (0: 112,000 bytes; scenes whose tiles need more
 *     are refused -- plan them with smaller tiles).
 *   submit: the scene must be started (start()) on the server's device and
 *     precision, with symplectic Euler and resident tiles and bins off
 *     (set_resident 0).  Its queued work is waited for; until poll reports
 *     the request done, the scene's own stepping, transfers and parameter
 *     changes return TITAN_GB300_ESTATE.  TITAN_GB300_EBUSY: no free slot.
 *     *ticket identifies the request.
 *   poll: TITAN_GB300_OK once the request is done (the scene's clock and
 *     step count have advanced by nsteps and it is usable again),
 *     TITAN_GB300_EBUSY while it runs, TITAN_GB300_ETIMEOUT if the kernel's
 *     bounded waits gave up (the server is then unusable).
 *   info: out[0] occupied slots, [1] free slots, [2] kernel launches so far,
 *     [3] the kernel's last status (1 running, 2 stopped, 3 left idle, 4
 *     timed out), [4] CTAs, [5] dynamic shared memory per CTA.
 *   destroy: a stop word ends the kernel at its next step boundary; scenes
 *     still in flight are released with an undefined state. */
typedef struct titan_gb300_server titan_gb300_server;
int titan_gb300_server_create(titan_gb300_server **out, int device, int precision, int max_slots,
                              int64_t tile_smem_bytes);
int titan_gb300_server_submit(titan_gb300_server *srv, titan_gb300_sim *sim, int64_t nsteps, int64_t *ticket);
int titan_gb300_server_poll(titan_gb300_server *srv, int64_t ticket);
int titan_gb300_server_info(const titan_gb300_server *srv, int64_t out[6]);
const char *titan_gb300_server_last_error(const titan_gb300_server *srv);
void titan_gb300_server_destroy(titan_gb300_server *srv);

/* CUDA stream (cudaStream_t) the handle queues work on. */
void *titan_gb300_stream(titan_gb300_sim *sim);

/* Plan figures for reports: out[0] masses, [1] springs, [2] tiles,
 * [3] slab entries, [4] halo slots, [5] incidence words, [6] heavy masses,
 * [7] dynamic shared memory bytes per CTA, [8] threads per CTA,
 * [9] algorithmic bytes per step, [10] implementation bytes per step
 * (tables and slabs as laid out), [11] actuated entries. */
int titan_gb300_plan_info(const titan_gb300_sim *sim, int64_t out[12]);

/* ---- host-only helpers (no GPU needed) ------------------------------------ */

/* Builds the tile plan of the current scene on the host only (no GPU work;
 * with tile_masses 0 the default tile reads the device's SM count, 152 when
 * there is no device), for inspection, validation and adopt_plan; start()
 * builds its own otherwise.  The planner runs on up to 16 host threads
 * (environment variable TITAN_GB300_PLAN_THREADS: another limit, 1 to 64);
 * the plan is the same for any thread count.  The tables are copied out
 * with titan_gb300_plan_table, which returns the element count (and copies
 * when out != NULL), or -1 for an unknown table. */
int titan_gb300_plan_host(titan_gb300_sim *sim, int tile_masses);
int64_t titan_gb300_plan_table(const titan_gb300_sim *sim, int table, void *out);
#define TITAN_GB300_T_NEW2OLD 0        /* int32: tiled index -> creation index   */
#define TITAN_GB300_T_TILE_MASS_OFF 1  /* int64: ntiles+1                        */
#define TITAN_GB300_T_TILE_HALO_OFF 2  /* int64: ntiles+1                        */
#define TITAN_GB300_T_HALO 3           /* int32: tiled indices of halo masses    */
#define TITAN_GB300_T_TILE_ENT_OFF 4   /* int64: ntiles+1                        */
#define TITAN_GB300_T_TILE_NACT 5      /* int32: actuated entries lead each slab */
#define TITAN_GB300_T_ENT_ENDS 6       /* uint32: left slot | right << 12 | type << 24 */
#define TITAN_GB300_T_ENT_SPRING 7     /* int64: spring of each entry            */
#define TITAN_GB300_T_TILE_WARP_OFF 8  /* int64: ntiles+1                        */
#define TITAN_GB300_T_WARP_INC_OFF 9   /* uint32: per warp, into INC             */
#define TITAN_GB300_T_DEG 10           /* uint8: per tiled mass, 255 = heavy     */
#define TITAN_GB300_T_INC 11           /* uint16: entry | 0x8000 for a left end  */
#define TITAN_GB300_T_TILE_HEAVY_OFF 12 /* int64: ntiles+1                       */
#define TITAN_GB300_T_HEAVY_LOCAL 13   /* uint16                                 */
#define TITAN_GB300_T_HEAVY_INC_OFF 14 /* uint32: nheavy+1                       */
#define TITAN_GB300_T_HEAVY_INC 15     /* uint16                                 */
#define TITAN_GB300_T_BODY_OF_TILE 16  /* int32                                  */
#define TITAN_GB300_T_TILE_NH 17       /* int32: halo masses of each tile (HALO lists are padded to 4) */
/* resident bins (set_resident): */
#define TITAN_GB300_T_RES_BIN_MASS_OFF 18 /* int64: nbins+1, into RES_MASS       */
#define TITAN_GB300_T_RES_BIN_WARP_OFF 19 /* int64: nbins+1, into RES_WARP_REC_OFF */
#define TITAN_GB300_T_RES_MASS 20      /* int32: tiled index of each resident mass */
#define TITAN_GB300_T_RES_BODY 21      /* int32: its body                        */
#define TITAN_GB300_T_RES_DEG 22       /* uint8: its degree (0 if fixed)         */
#define TITAN_GB300_T_RES_ACT_MASK 23  /* uint64: bit j = record j is actuated   */
#define TITAN_GB300_T_RES_WARP_REC_OFF 24 /* uint32: first record of each bin warp */
#define TITAN_GB300_T_RES_WORDS 25     /* uint32: other (bin-local) | 0x8000 if right end | type << 16 */
#define TITAN_GB300_T_RES_REC_SPRING 26 /* int64: spring of each record, -1 = padding */
#define TITAN_GB300_T_RES_RESIDENT 27  /* uint8: per body, 1 if resident         */

/* Lattice builder of createLattice (src/sim.cu:1923-1944, src/object.cu:232-293):
 * fills pos (3*nx*ny*nz) and, when non-NULL, left/right/rest of the
 * titan_gb300_lattice_springs(nx,ny,nz) springs, in the reference's order. */
/* Point-in-mesh test of STL import on GPU `device` (stl::stlFile::inside,
 * include/Titan/stlparser.h:213-276, for Simulation::importFromSTL,
 * src/sim.cu:1855-1921): inside[i] = 1 when more than half of num_rays rays
 * from point i cross the triangles an odd number of times.  Rays come from a
 * counter-based generator keyed by seed, point and ray (the reference uses
 * rand()), so the result is reproducible.  tri: 9 doubles per triangle
 * (v1, v2, v3); pts: 3 per point; num_rays in [1, 64].  Blocking. */
int titan_gb300_stl_inside(int device, const double *tri, int64_t ntri, const double *pts, int64_t npts,
                           int num_rays, uint64_t seed, uint8_t *inside);

int64_t titan_gb300_lattice_springs(int nx, int ny, int nz);
int titan_gb300_lattice(const double center[3], const double dims[3], int nx, int ny, int nz,
                        double *pos, int32_t *left, int32_t *right, double *rest);

/* Version string of this library. */
const char *titan_gb300_version(void);

#ifdef __cplusplus
}
#endif
#endif
