/*
 * svm.h — C ABI of the GB300 spherical vertex-model step (libsvm.so).
 *
 * This is the drop-in boundary for the hot path of DanielMSussman/curvedSpaceVertexModel:
 * per-cell spherical-polygon geometry, the quadratic area/perimeter vertex forces, T1 edge
 * flips, the Brownian and FIRE updaters with renormalisation onto the sphere, and the
 * sphere's cell list.  In the reference these are reached through the model/updater classes
 * and the free `gpu_*` launcher functions declared in its .cuh headers; each entry point below
 * cites the reference interface it replaces (paths relative to the reference repository).
 *
 * Conventions
 *   - Every function returns an int status (SVM_OK == 0) and never throws.
 *   - A model owns its device arrays and a CUDA stream; all device work is ordered on that
 *     stream.  Functions that take or return host arrays synchronise that stream.
 *   - Host arrays use the reference's layouts: positions and vectors are AoS double[3*n];
 *     rings are row-major int[nCells*ringStride] in clockwise order seen from outside with
 *     ringCounts[nCells]; vertex->cell and vertex->vertex lists are int[3*nVertices];
 *     area/perimeter pairs are double[2*nCells] (area first).
 *   - Device-side failures (a ring outgrowing its capacity, a full T1 work list, a cell-list
 *     bin overflow, a bounded wait that ran out) set bits in a device status word instead of
 *     trapping; svm_model_status() reads and clears it.
 */
#ifndef SVM_H
#define SVM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------------------- */
#define SVM_OK 0
#define SVM_ERR_ARG 1          /* invalid argument or handle */
#define SVM_ERR_CUDA 2         /* CUDA runtime error (launch, copy, allocation) */
#define SVM_ERR_HULL 3         /* degenerate or invalid convex hull */
#define SVM_ERR_DEVICE 4       /* device status word non-zero; see SVM_DEV_* bits */
#define SVM_ERR_NO_DEVICE 5    /* no CUDA device */

/* device status word bits (svm_model_status) */
#define SVM_DEV_RING_OVERFLOW 0x1   /* a T1 would grow a ring beyond its capacity */
#define SVM_DEV_T1_OVERFLOW 0x2     /* T1 bookkeeping capacity exceeded */
#define SVM_DEV_CELLLIST_OVERFLOW 0x4 /* more points in a bin than the slot table holds */
#define SVM_DEV_BAD_TOPOLOGY 0x8    /* an edge's cells could not be classified */
#define SVM_DEV_T1_TIMEOUT 0x10     /* a grid barrier of the multi-block T1 pass gave up waiting
                                       (the state of that pass is undefined) */

/* Noise sources of the Brownian step. */
#define SVM_NOISE_PHILOX 0     /* in-kernel counter-based Philox4x32-10 bits, ziggurat normals */
#define SVM_NOISE_BUFFER 1     /* standard normals supplied by the caller, vertex-major [3*Nv] */

/* FIRE stopping criteria. */
#define SVM_FIRE_RMS_OVER_N 0  /* the reference's sqrt(sum_i |F_i|^2) / N (energyMinimizerFIRE.cpp:140) */
#define SVM_FIRE_MAX_FORCE 1   /* max_i |F_i| */

const char* svm_status_string(int status);
int svm_device_count(int* count);

/* Cell centres of the reference's initialisation: n points uniform on the unit sphere drawn from
 * std::mt19937(seed) through std::uniform_real_distribution<double> (theta = acos(2v-1),
 * phi = 2 pi u; sphericalModel::setParticlePositionsRandomly, src/model/sphericalModel.cpp:37-51),
 * then scaled to R = sqrt(n / 4 pi) (sphericalVertexModel.cpp:12).  seed < 0 keeps the default
 * engine seed 13377 (src/utilities/noiseSource.h:24).  out: double[3n]. */
int svm_random_cell_centres(int seed, int n, double* out);
/* Initial directors for the given vertex positions (one unit tangent vector per vertex, made as
 * sphericalVertexModel.cpp:58-70 makes them) drawn from the seeded stream after the cell centres
 * and the cell model's directors: out[3 nV].  The reference draws them from the model's own
 * default noise source, seeded by random_device (noiseSource.h:21-30), so its directors do not
 * repeat between runs; these do, with the same distribution. */
int svm_random_vertex_directors(int seed, int nCells, const double* vertexPos, int nV, double* out);

/* ---- initial topology (host) ------------------------------------------------------------
 * Replaces convexHullCGALInterface::sphericalConvexHullForVertexModel
 * (src/model/convexHullCGAL.cpp:82-186): hull of the cell centres, one vertex per facet at the
 * normalised facet centroid, CCW vertex->cell / vertex->vertex slots, clockwise cell rings. */
typedef struct svm_topology svm_topology;
int svm_topology_from_points(const double* cellCentres, int nCells, svm_topology** out);
/* The same topology computed on the device (cell centres: HOST double[3*nCells]): per-centre
 * stars of the hull by gift wrapping over cell-list candidates, certified by their circumcaps,
 * checked for consistency, then numbered and assembled exactly as svm_topology_from_points does.
 * Replaces convexHullCGALInterface::sphericalConvexHullForVertexModel (convexHullCGAL.cpp:82-186).
 * SVM_ERR_HULL when the stars do not close into one triangulated sphere, or when a centre would need
 * more than 512 candidates (a local density roughly 7x the mean): svm_topology_from_points then
 * builds the same topology on the host. */
int svm_topology_from_points_gpu(const double* cellCentres, int nCells, void* stream, svm_topology** out);
/* Same contract from caller-supplied hull triangles (CCW seen from outside, int[3*nTri]). */
int svm_topology_from_triangles(const double* cellCentres, int nCells, const int* triangles, int nTriangles,
                                svm_topology** out);
int svm_topology_sizes(const svm_topology* t, int* nCells, int* nVertices, int* maxRing);
int svm_topology_get(const svm_topology* t, double* vertexPos, int* rings, int ringStride,
                     unsigned* ringCounts, int* vertexCells, int* vertexNeighbors);
void svm_topology_free(svm_topology* t);

/* ---- model ---------------------------------------------------------------------------------
 * Device-resident state of sphericalVertexModel (src/model/sphericalVertexModel.h:10-123).
 * ringCapacity is the initial per-cell ring capacity; it grows on demand as the reference's ring
 * width does (sphericalVertexModel.cpp:733-758; svm_model_set_ring_headroom below).  stream may
 * be NULL (the model then creates its own stream). */
typedef struct svm_model svm_model;
int svm_model_create(int nCells, int nVertices, int ringCapacity, double radius, void* stream, svm_model** out);
int svm_model_destroy(svm_model* m);
/* Arithmetic of the step (no counterpart in the reference, whose scalar type is fixed at compile
 * time, inc/std_include.h:49-78):
 *   SVM_PRECISION_FP64  - the plain form: every quantity in FP64 (default);
 *   SVM_PRECISION_MIXED - FP32 positions, forces and integration, with the included angles and
 *                         the spherical-excess areas, the energy accumulation and the
 *                         renormalisation onto the sphere in FP64;
 *   SVM_PRECISION_FP64_VECTOR - FP64 throughout, with the forces evaluated as the exact energy
 *                         gradient in vectors of position differences instead of the reference's
 *                         closed forms in spherical coordinates (sphericalDomain.h:248-411), whose
 *                         triangle term loses digits on nearly degenerate centroid-fan triangles
 *                         and floors max|F| near 1e-8 at N = 20k.  For minimisation to tight force
 *                         tolerances.
 * Switching converts the current positions.  FIRE runs in the two FP64 forms. */
#define SVM_PRECISION_FP64 0
#define SVM_PRECISION_MIXED 1
#define SVM_PRECISION_FP64_VECTOR 2
int svm_model_set_precision(svm_model* m, int precision);

/* Upload topology and positions (host arrays, reference layouts). */
int svm_model_set_topology(svm_model* m, const double* vertexPos, const int* rings, int ringStride,
                           const unsigned* ringCounts, const int* vertexCells, const int* vertexNeighbors);
/* setPreferredParameters (sphericalVertexModel.cpp:103-109) and a per-cell variant. */
int svm_model_set_preferred_parameters(svm_model* m, double a0, double p0);
int svm_model_set_preferred_array(svm_model* m, const double* a0p0);
/* setScalarModelParameter (Kr = K_A/K_P, sphericalVertexModel.h:85) */
int svm_model_set_scalar_model_parameter(svm_model* m, double kr);
/* setT1Threshold (sphericalVertexModel.h:87) */
int svm_model_set_t1_threshold(svm_model* m, double threshold);
/* simpleModel::restrictedMotion (src/model/simpleModel.h:145): no T1 when non-zero */
int svm_model_set_restricted_motion(svm_model* m, int restricted);

/* computeGeometry -> gpu_spherical_vertex_model_geometry (sphericalVertexModel.cuh:21-35),
 * with the CPU path's total-area check and triangle fallback (sphericalVertexModel.cpp:304-310). */
int svm_model_compute_geometry(svm_model* m);
/* computeForces -> gpu_quadratic_spherical_cellular_force (sphericalVertexModel.cuh:37-51). */
int svm_model_compute_forces(svm_model* m);
/* computeEnergy (sphericalVertexModel.cpp:150-160): sum_c Kr (A-A0)^2 + (P-P0)^2; synchronises. */
int svm_model_compute_energy(svm_model* m, double* energy);
/* moveParticles -> gpu_move_particles_on_sphere (sphericalVertexModel.cuh:14-19) followed by
 * enforceTopology unless motion is restricted.  disp is a DEVICE pointer to double[3*Nv]. */
int svm_model_move_particles(svm_model* m, const double* dispDevice, double scale);
/* Same with a host displacement array (copied on the model's stream). */
int svm_model_move_particles_host(svm_model* m, const double* disp, double scale);
/* enforceTopology -> gpu_vm_test_edges_for_T1 + gpu_vm_parse_multiple_flips + gpu_vm_flip_edges
 * (sphericalVertexModel.cuh:53-93), with the CPU path's sequential flip order. */
int svm_model_enforce_topology(svm_model* m);

/* Host getters/setters (synchronise). */
int svm_model_get_positions(svm_model* m, double* out);
int svm_model_set_positions(svm_model* m, const double* in);
int svm_model_get_forces(svm_model* m, double* out);
int svm_model_get_velocities(svm_model* m, double* out);
int svm_model_set_velocities(svm_model* m, const double* in);
int svm_model_get_area_perimeter(svm_model* m, double* out);
int svm_model_get_cell_positions(svm_model* m, double* out);
int svm_model_get_rings(svm_model* m, int* rings, int ringStride, unsigned* ringCounts);
/* Ring capacity.  growCellVerticesList (src/model/sphericalVertexModel.cpp:733-758, called from the
 * T1 passes at :492 and :824) widens the reference's ring storage when a flip would fill a ring.
 * Here every T1 pass records its largest ring, and before a pass (between replays of 8 steps for
 * svm_brownian_run, between batches of 32 iterations for svm_fire_minimize) the capacity grows --
 * the rings re-laid out at a width that is a multiple of 4 -- whenever `slots` or fewer are free in
 * the largest ring (default 2).  The width changes no result.  The host waits for the pass before
 * last before launching a pass, so its reading lags at most two passes (16 steps of
 * svm_brownian_run); a flip that still finds its ring full is refused and sets
 * SVM_DEV_RING_OVERFLOW.  svm_model_ring_info: capacity, largest ring count, growths so far. */
int svm_model_set_ring_headroom(svm_model* m, int slots);
int svm_model_ring_info(svm_model* m, int* out3);
int svm_model_get_vertex_cells(svm_model* m, int* out);
int svm_model_get_vertex_neighbors(svm_model* m, int* out);
/* The last geometry pass's total-area check (sphericalVertexModel.cpp:304-310): sum of cell
 * areas, its excess over 4 pi R^2, and whether the triangle-fan fallback replaced the areas. */
int svm_model_area_check(svm_model* m, double* totalArea, double* excess, int* fallbackTaken);
/* Geometry passes of a single sphere that took the triangle-fan fallback since the last call
 * (read and cleared). */
int svm_model_fallback_count(svm_model* m, int* count);
/* Device status word (SVM_DEV_* bits); read and cleared. */
int svm_model_status(svm_model* m, int* deviceStatus);
/* T1 flips performed since the last call, as (vertex1, vertex2) pairs in the order they were
 * applied; *count receives the total (pairs beyond `capacity` are dropped). */
int svm_model_take_flips(svm_model* m, int* pairs, int capacity, int* count);
/* T1 statistics accumulated since the last call (then cleared), 6 ints: passes, edges flagged by
 * the test, edges that ran in the parallel rounds, flips, parallel rounds, passes replayed one flip
 * at a time after a rollback.  (The reference's T1 loop keeps no such counters.) */
int svm_model_t1_stats(svm_model* m, int* stats6);
/* SM cycles spent by the first segment of the parallel T1 pass in its phases since the last call
 * (extraction of the flagged edges, reservation, flips, release, end), when cycles5 is non-NULL
 * and the counters are on; then (re)arms them (enable != 0) or turns them off. */
int svm_model_t1_clocks(svm_model* m, int enable, unsigned long long* cycles5);
/* Blocks of a single sphere's parallel T1 pass: 0 = automatic (a cooperative grid of about one
 * block per 3000 vertices from 20000 vertices on, else one block), 1 = one block, n > 1 = a
 * cooperative grid of n blocks (capped at the device's co-resident count).  Performance only:
 * the flips and every later value are the same for any count.  Ignored by batches. */
int svm_model_set_t1_blocks(svm_model* m, int blocks);
/* Polls of each grid-barrier wait of a cooperative T1 pass before it gives up (default 2^20, at
 * least 67 ms).  A wait that runs out sets SVM_DEV_T1_TIMEOUT and ends the kernel: the pass is then
 * incomplete and the model's topology is not to be trusted (recreate it).  No counterpart in the
 * reference (its T1 loop runs on one CPU thread); a diagnostic hook, e.g. to check that an
 * exhausted wait is reported rather than hung. */
int svm_model_set_t1_wait_limit(svm_model* m, int polls);
int svm_model_synchronize(svm_model* m);
/* Dynamical observables of the cell positions (dynamicalFeatures, src/analysis/dynamicalFeatures.cpp):
 * svm_model_set_dynamics_reference snapshots the current cell positions (as computed by the last
 * geometry pass) on the device; svm_model_dynamics returns, over the first floor(N fraction)
 * cells, the mean squared geodesic displacement from them (NaN distances skipped) and the fraction
 * of cells displaced by less than `cutoff` (the reference's default 0.5). */
int svm_model_set_dynamics_reference(svm_model* m);
int svm_model_dynamics(svm_model* m, double fraction, double cutoff, double* msd, double* overlap);
/* Directors (one per vertex, simpleModel.h:104-113) of a single sphere: host double[3 Nv] in or out. */
int svm_model_set_directors(svm_model* m, const double* dirs);
int svm_model_get_directors(svm_model* m, double* dirs);
/* One self-propelled-particle step (sphericalSelfPropelledParticle::integrateEOMCPU,
 * src/updaters/sphericalSelfPropelledParticle.cpp:16-47) of a single FP64 sphere: forces,
 * disp = dt (v0 n + mu F), move with T1 unless restricted, then each director projected onto the
 * tangent plane, normalised and rotated about its vertex's position vector by
 * r sqrt(2 dt tau), r uniform in [-1/2, 1/2): SVM_NOISE_BUFFER takes the Nv draws from `uniforms`
 * (host), SVM_NOISE_PHILOX draws them in-kernel from (seed, step counter, vertex). */
int svm_spp_step(svm_model* m, double dt, double mu, double v0, double tau, int noiseMode, const double* uniforms,
                 uint64_t seed);
/* One step of sphericalVectorialVicsek (src/updaters/sphericalVectorialVicsek.cpp:5-60) on the
 * vertex model, whose neighbours are each vertex's three vertex neighbours: forces, the
 * self-propelled move dt (v0 n + mu F) with its T1 flips, then per vertex the target
 * (n + neighbours' n) / 4 + eta xi (xi a random unit vector projected onto the tangent plane and
 * normalised), projected and normalised, and n += (dt / tau)(target - n), projected and
 * normalised.  noiseMode SVM_NOISE_BUFFER: `uniforms` = HOST double[2 nV], (u, w) per vertex in
 * [0, 1) as the reference draws them; SVM_NOISE_PHILOX: in-kernel draws (seed, step).  FP64 form,
 * single spheres; tau must be non-zero (SVM_ERR_ARG). */
int svm_vicsek_step(svm_model* m, double dt, double mu, double v0, double eta, double tau, int noiseMode,
                    const double* uniforms, uint64_t seed);
/* Device pointer of the current positions for callers that keep data on the GPU: double4 (x, y,
 * z, unused) per vertex in the FP64 form, float4 in the mixed form.  Valid until the next step,
 * precision switch or svm_model_destroy. */
int svm_model_device_positions(svm_model* m, void** ptr);
/* The CUDA stream (cudaStream_t) all of the model's work is ordered on. */
int svm_model_stream(svm_model* m, void** stream);

/* Per-phase CUDA-event timing on the model's stream (the GPU counterpart of the reference's
 * geoProf / forceProf / moveProf profilers, sphericalVertexModel.h:87-89 and
 * src/utilities/profiler.h:8-45).  While enabled, every launch of a phase outside graph capture
 * is bracketed by events; svm_model_profile_read synchronises and returns, per phase, the total
 * milliseconds and the number of kernel launches since the last read.  Phases: */
#define SVM_PHASE_CORNERS 0    /* per-vertex corner arcs/angles (+ fused T1 edge test) */
#define SVM_PHASE_CELLS 1      /* per-cell centroid, area, perimeter, total-area check */
#define SVM_PHASE_FALLBACK 2   /* triangle-fan area fallback */
#define SVM_PHASE_FORCE 3      /* forces (+ fused Brownian integrate and move, or FIRE half-kick) */
#define SVM_PHASE_T1APPLY 4    /* ordered T1 flips (parallel pass, sequential replay, patch: 3 kernels) */
#define SVM_PHASE_MOVE 5       /* standalone moves and velocity-Verlet drift */
#define SVM_PHASE_COUNT 6
/* enable: 0 off, 1 every phase; SVM_PROFILE_ONLY | (1 << phase) | ... brackets only the phases named
 * (each pair of events adds a little time to the step) and counts the launches of all of them. */
#define SVM_PROFILE_ONLY 0x100
int svm_model_profile(svm_model* m, int enable);
int svm_model_profile_read(svm_model* m, double* msPerPhase, int* launchesPerPhase);

/* ---- allocation-free energy -----------------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory — hosts whose
 * device memory belongs entirely to their own pool allocator, and per-step code that must not pay
 * cudaMalloc's implicit device-wide synchronisation — this computes
 * energy = sum_c Kr (A_c - A0_c)^2 + (P_c - P0_c)^2 (the quantity of svm_model_compute_energy)
 * from caller-owned DEVICE arrays areaPerimeter[2*nCells] and preference[2*nCells] into the DEVICE
 * double *energy, on `stream` (NULL: the legacy default stream), without allocating.  Its scratch is
 * one static device array in libsvm of SVM_NOALLOC_MAX_CELLS / 256 + 32 doubles (64 KB) per device;
 * nCells above SVM_NOALLOC_MAX_CELLS returns SVM_ERR_ARG.  Every call on a device shares that
 * array (it keeps the last call's contents; the part that must start at zero is cleared on
 * `stream` before each launch), so calls that overlap on the GPU race.  The first call on each
 * device looks up the array's address (cudaGetSymbolAddress, with that device current); make that
 * first call before any stream capture. */
#define SVM_NOALLOC_MAX_CELLS 2097152
int svm_energy_noalloc(const double* areaPerimeter, const double* preference, double kr, int nCells,
                       double* energy, void* stream);

/* ---- Brownian dynamics ---------------------------------------------------------------------
 * brownianDynamics::integrateEOMGPU (src/updaters/brownianDynamics.cpp:14-27) ->
 * gpu_brownian_eom_integration (brownianDynamics.cuh:15-22): forces, then
 * disp = sqrt(2 dt mu T) xi + dt mu F, then moveParticles.  One call = one timestep.
 * noiseMode SVM_NOISE_BUFFER reads standard normals from noise (DEVICE pointer, [3*Nv]);
 * SVM_NOISE_PHILOX draws them in-kernel from (seed, the model's step counter, vertex). */
int svm_brownian_step(svm_model* m, double T, double dt, double mu, int noiseMode, const double* noiseDevice,
                      uint64_t seed);
/* Same with host-supplied standard normals (copied on the model's stream). */
int svm_brownian_step_host_noise(svm_model* m, double T, double dt, double mu, const double* noise);
/* One timestep with Philox noise and host buffers, in one stream sequence with one
 * synchronisation: positions[3 nV] uploaded from posIn (NULL: keep the device state), the step,
 * *energyOut = the energy of the geometry the step's forces used (what svm_model_compute_energy
 * returns after a step; computeEnergy, sphericalVertexModel.cpp:150-160), and the new positions
 * in posOut (NULL: none).  Pinned host buffers make the upload asynchronous DMA; in the FP64 forms
 * a page-locked (mapped) posOut is written by the step's own kernels -- the force kernel as it
 * moves the vertices, the T1 pass for the vertices its flips move -- so no copy follows the step. */
int svm_brownian_step_io(svm_model* m, double T, double dt, double mu, uint64_t seed, const double* posIn,
                         double* posOut, double* energyOut);
/* nSteps timesteps with Philox noise, launched as a captured CUDA graph. */
int svm_brownian_run(svm_model* m, double T, double dt, double mu, uint64_t seed, int nSteps);

/* ---- FIRE ----------------------------------------------------------------------------------
 * energyMinimizerFIRE (src/updaters/energyMinimizerFIRE.{h,cpp}) over velocityVerlet
 * (src/updaters/velocityVerlet.cpp:40-59): setFIREParameters (energyMinimizerFIRE.cpp:203-214),
 * minimize (180-200).  Reductions and the dt/alpha control run on the device. */
typedef struct svm_fire svm_fire;
int svm_fire_create(svm_model* m, double dt, double alphaStart, double dtMax, double dtInc, double dtDec,
                    double alphaDec, int nMin, double forceCutoff, double alphaMin, int maxIterations,
                    svm_fire** out);
/* A minimizer may outlive its model: svm_model_destroy detaches it, after which minimize and
 * state return SVM_ERR_ARG and destroy only frees it. */
int svm_fire_destroy(svm_fire* f);
/* Runs until the criterion drops to forceCutoff or maxIterations; returns the iterations done
 * by this call and the final value of the criterion. */
int svm_fire_minimize(svm_fire* f, int criterion, int* iterations, double* criterionValue);
/* setMaximumIterations (energyMinimizerFIRE.h:37): the cap on the total iteration count, keeping
 * dt, alpha and the counters (a later minimize continues from there). */
int svm_fire_set_max_iterations(svm_fire* f, int maxIterations);
/* state: dt, alpha, power, rms_over_n, max_force, n_since, iterations (7 doubles). */
int svm_fire_state(svm_fire* f, double* state7);

/* ---- per-phase FIRE and velocity Verlet ------------------------------------------------------
 * The pieces minimize strings together, for callers that drive their own loop.  All run on the
 * model's stream in the FP64 forms (SVM_ERR_ARG in the mixed form); masses are 1, as the model's are.
 *
 * fireStep (src/updaters/energyMinimizerFIRE.h:56, fireStepCPU energyMinimizerFIRE.cpp:122-174):
 * on the model's current forces and velocities, P = sum F.v, |F|^2, |v|^2 and max |F|; the velocity
 * update v <- (1 - alpha) v + alpha |v|/|F| F (v <- 0 when P <= 0) and the dt / alpha adaptation.
 * The sums run in the same blocks and order as a minimize iteration's, so a loop of
 * svm_velocity_verlet_step(m, dt, 1) with dt = state[0] and svm_fire_step equals minimize bit for
 * bit; like fireStep it does not count an iteration (minimize does, cpp:191). */
int svm_fire_step(svm_fire* f);
/* velocityVerlet::integrateEquationOfMotion (src/updaters/velocityVerlet.cpp:40-59, CPU 6-38),
 * nSteps times: disp = dt v + (dt^2 / 2) F and v += (dt / 2) F (gpu_displacement_velocity_verlet,
 * velocityVerlet.cuh:21-28), the move onto the sphere with T1 flips unless motion is restricted
 * (moveParticles), geometry and forces (sim->computeForces), v += (dt / 2) F (gpu_update_velocity).
 * Forces must be current on entry (svm_model_compute_forces), as in the reference. */
int svm_velocity_verlet_step(svm_model* m, double dt, int nSteps);
/* gpu_update_velocity (src/updaters/velocityVerlet.cuh:14-19): v += (dt / 2) F / m. */
int svm_vv_half(svm_model* m, double dt);
/* gpu_dVec_dot_products (src/utilities/utilities.cuh:74) over the model's forces F and velocities v:
 * out4 = (sum F.v, sum F.F, sum v.v, max |F|), block sums in a fixed order; synchronises. */
int svm_reduce_dots(svm_model* m, double* out4);

/* ---- cell list -----------------------------------------------------------------------------
 * hyperrectangularCellList (src/utilities/hyperrectangularCellList.{h,cpp}): cubic grid over
 * [-radius, radius]^3 with side count floor(2 radius / a) made even, bin_d = floor((x_d +
 * radius) / h).  Points of a bin are listed in ascending index, as computeCPU does (165-214). */
typedef struct svm_cell_list svm_cell_list;
int svm_cell_list_create(double a, double radius, int nPoints, int slotCapacity, void* stream, svm_cell_list** out);
int svm_cell_list_destroy(svm_cell_list* cl);
/* Bins the model's current vertex positions (computeCellList -> gpu_compute_cell_list,
 * hyperrectangularCellList.cuh:18-30). */
int svm_cell_list_compute_model(svm_cell_list* cl, svm_model* m);
/* Bins caller points (DEVICE double[3*n] AoS). */
int svm_cell_list_compute(svm_cell_list* cl, const double* pointsDevice, int n);
/* nside, Nmax (the reference's grow-only width), per-bin counts [nside^3] and the slot table
 * [nside^3 * Nmax] (ascending point index, -1 past the count); synchronises. */
int svm_cell_list_get(svm_cell_list* cl, int* nside, int* nmax, unsigned* counts, int* slots, long slotsCapacity);
int svm_cell_list_bins(svm_cell_list* cl, int* binOfPoint);

/* ---- neighbour list ------------------------------------------------------------------------
 * neighborList (src/utilities/neighborList.{h,cpp}; the spherical model builds it with range 1 and
 * radius R + 2.5, sphericalModel.cpp:21): a cell list of grid size range / subGridReduction over
 * [-radius, radius]^3 (slotCapacity slots per bin to start with; a bin that overflows them widens
 * every bin, as the reference's cell list grows its Nmax), then per point every other point at
 * minimum-image distance below `range` in a periodic box of side 2 radius, listed in the order of
 * the adjacent bins (computeAdjacentCells) and of each bin's slots.  Nmax starts at 4 and grows to
 * the largest count (the list is recomputed then).  Points must lie in [-radius, radius)^3: one
 * outside (or not finite) returns SVM_ERR_DEVICE.  Replaces neighborList::computeNeighborLists
 * (neighborList.h:17-28) and its launcher gpu_compute_neighbor_list (neighborList.cuh). */
typedef struct svm_neighbor_list svm_neighbor_list;
int svm_neighbor_list_create(double range, double radius, int subGridReduction, int nPoints, int slotCapacity,
                             void* stream, svm_neighbor_list** out);
int svm_neighbor_list_destroy(svm_neighbor_list* nl);
/* Caller points (DEVICE double[3*n] AoS), or the model's current vertex positions. */
int svm_neighbor_list_compute(svm_neighbor_list* nl, const double* pointsDevice, int n);
int svm_neighbor_list_compute_model(svm_neighbor_list* nl, svm_model* m);
/* Nmax; per point the neighbour count [n]; per (point, k < Nmax), k-major within a point: index,
 * displacement (3 doubles) and distance, zero past the count (capacity >= n Nmax entries). */
int svm_neighbor_list_get(svm_neighbor_list* nl, int* nmax, unsigned* npp, int* idx, double* vec, double* dist,
                          long capacity);

/* ---- batches of replicas -------------------------------------------------------------------
 * No counterpart in the reference, which runs one sphere per process (its seed loops,
 * minimization.cpp:98-132, run instances one after another).  A batch is one svm_model holding
 * nReplicas independent spheres back to back: replica r has nCells[r] cells (cells
 * [cellOff[r], cellOff[r+1])), nVertices[r] = 2 nCells[r] - 4 vertices (vertices
 * [vertOff[r], vertOff[r+1])) and radius radius[r].  Every svm_model_* call applies to the whole
 * batch; rings, vertex lists and per-cell arrays passed to them use global indices, and per-cell
 * (A0, P0) (svm_model_set_preferred_array) sweeps P0 across replicas.  Batches run the
 * mixed-precision form (switching to FP64 returns SVM_ERR_ARG).  A Brownian step (svm_brownian_step
 * or _run) of a batch uses the per-replica temperatures of svm_batch_set_temperatures (default 0;
 * its T argument is ignored), the area check is per replica, and each replica's T1 flips are the
 * ones the single-sphere loop would make. */
int svm_batch_create(int nReplicas, const int* nCells, const int* nVertices, int ringCapacity, const double* radius,
                     void* stream, svm_model** out);
int svm_batch_replicas(svm_model* m, int* nReplicas);
/* cellOffsets, vertexOffsets: nReplicas + 1 ints each (either may be NULL). */
int svm_batch_offsets(svm_model* m, int* cellOffsets, int* vertexOffsets);
int svm_batch_set_temperatures(svm_model* m, const double* temperatures);
/* Per-replica energy sum_c Kr (A - A0)^2 + (P - P0)^2 of the current geometry. */
int svm_batch_energies(svm_model* m, double* energies);
/* Per-replica total area, excess over 4 pi R^2 and fallback flag of the last geometry. */
int svm_batch_area_check(svm_model* m, double* totals, double* excess, int* fallbackTaken);
/* Autotuning of the block size of the batch's corner, cell and force kernels, one KernelTuner
 * each over block sizes lo, lo+step, ..., hi (multiples of 32, at most 1024, and at most the
 * largest block each kernel's register use allows): the reference's
 * kernelTuner(start, end, step, nSamples, period) (src/utilities/kernelTuner.{h,cpp}).  While a
 * tuner samples, svm_brownian_run runs steps one by one with those kernels timed; graph-replayed
 * steps count as untimed calls toward the rescan period.  lo <= 0 turns tuning off (block 256). */
int svm_batch_autotune(svm_model* m, int lo, int hi, int step, int nSamples, int period);
/* Current block sizes (corners, cells, force) and whether the initial sampling is complete. */
int svm_batch_block_sizes(svm_model* m, int* sizes3, int* samplingComplete);

/* ---- kernel tuner ----------------------------------------------------------------------------
 * kernelTuner (src/utilities/kernelTuner.{h,cpp}) over CUDA events on `stream`: bracket a launch
 * with begin/end (end synchronises when the call is timed) and use svm_tuner_parameter for the
 * next launch.  svm_tuner_record feeds a time measured by other means (one end() call). */
typedef struct svm_tuner svm_tuner;
int svm_tuner_create(int start, int end, int step, int nSamples, int period, void* stream, svm_tuner** out);
int svm_tuner_destroy(svm_tuner* t);
int svm_tuner_begin(svm_tuner* t);
int svm_tuner_end(svm_tuner* t);
int svm_tuner_record(svm_tuner* t, float milliseconds);
int svm_tuner_parameter(svm_tuner* t, int* value);
int svm_tuner_sampling_complete(svm_tuner* t, int* complete);
/* candidates and their median times (printTimingData, kernelTuner.h:25-32) */
int svm_tuner_timing_data(svm_tuner* t, int* candidates, float* medians, int capacity, int* count);

/* ---- learned warm start for FIRE ------------------------------------------------------------
 * No counterpart in the reference.  A per-vertex MLP 24 -> 64 -> 64 -> 2 (ReLU, BF16 weights,
 * FP32 accumulation) reads the local tangent-frame geometry of a vertex (offsets to its three
 * neighbours and three cell centroids, the cells' A - A0, P - P0 and ring sizes, the force) and
 * predicts its displacement to the relaxed state in that frame.  Weights: FP32 master copy of
 * svm_mlp_parameter_count floats (W1[64][24], b1, W2[64][64], b2, W3[2][64], b3), Adam on the
 * master copy, forward on its BF16 rounding. */
typedef struct svm_mlp svm_mlp;
int svm_mlp_create(unsigned seed, void* stream, svm_mlp** out);
int svm_mlp_destroy(svm_mlp* mlp);
int svm_mlp_parameter_count(int* count);
int svm_mlp_set_weights(svm_mlp* mlp, const float* weights);   /* host; resets Adam */
int svm_mlp_get_weights(svm_mlp* mlp, float* weights);         /* host */
/* multiplies the network output into a displacement (the training targets' unit) */
int svm_mlp_set_output_scale(svm_mlp* mlp, double scale);
/* Features of every vertex of an FP64 model after geometry and forces: DEVICE float[24 nV], and
 * optionally the frames (e1, e2) as DEVICE double[6 nV]. */
int svm_mlp_features(svm_model* m, float* featuresDevice, double* framesDevice);
/* Gradient of mean_i |y_i - t_i|^2 over n samples (DEVICE X[24 n], T[2 n]) into HOST grad, and
 * the loss. */
int svm_mlp_gradient(svm_mlp* mlp, const float* X, const float* T, int n, float* grad, double* loss);
/* One epoch: Adam steps over mini-batches of `batch` samples taken in the DEVICE order[n]. */
int svm_mlp_train(svm_mlp* mlp, const float* X, const float* T, const int* order, int n, int batch,
                  float learningRate, double* meanLoss);
int svm_mlp_predict(svm_mlp* mlp, const float* X, int n, float* Y);   /* DEVICE arrays */
/* Fused inference on an FP64 model: geometry and forces, then per vertex features -> network ->
 * move by outputScale * (y0 e1 + y1 e2) onto the sphere (all vertices from the same state). */
int svm_mlp_warm_start(svm_mlp* mlp, svm_model* m);

/* ---- diagnostics ---------------------------------------------------------------------------
 * The FP64 kernels compute their divisions and square roots with integer-pipe IEEE arithmetic
 * (csrc/svm_softf64.cuh; no counterpart in the reference), and the FP32-bulk form's float <-> double
 * conversions likewise.  svm_softf64_check runs that device code against the hardware's correctly
 * rounded instructions on `cases` random operands per operation and returns the mismatches of
 * multiply, add, divide, square root, widening and narrowing (all zero). */
int svm_softf64_check(long long cases, unsigned long long seed, unsigned long long* mismatches6);

#ifdef __cplusplus
}
#endif
#endif /* SVM_H */
