/*
 * pbf103.h -- C ABI of the GB300-native Position Based Fluids step.
 *
 * Drop-in boundary for the reference solver API of DusanCojic/Fluid-Simulator
 * (class PBFSolver, include/pbf/pbf_solver.hpp:13-70).  Every entry point takes
 * plain pointers and sizes and returns a pbf_status whose values map 1:1 onto
 * the C++ exception types the reference throws; pbf_last_error() gives the
 * message.  The header-only C++ shim include/pbf103/pbf_solver.hpp rethrows
 * them as those exception types.
 *
 * Threading: one solver handle must not be used from two threads at once
 * (the reference class is not thread-safe either).  Every call that returns
 * data to the host is synchronous; pbf_step/pbf_run are synchronous too, like
 * PBFSolver::step (src/pbf/pbf_solver.cu:327).
 */
#ifndef PBF103_H
#define PBF103_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes <-> exception types thrown by the reference. */
typedef enum pbf_status {
    PBF_OK = 0,
    PBF_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument */
    PBF_ERR_LOGIC = 2,            /* std::logic_error (use before initialize) */
    PBF_ERR_OUT_OF_RANGE = 3,     /* std::out_of_range */
    PBF_ERR_LENGTH = 4,           /* std::length_error */
    PBF_ERR_OVERFLOW = 5,         /* std::overflow_error (neighbour capacity) */
    PBF_ERR_RUNTIME = 6           /* std::runtime_error (CUDA error, collisions did not converge) */
} pbf_status;

typedef struct pbf_float3 { float x, y, z; } pbf_float3;
typedef struct pbf_float4 { float x, y, z, w; } pbf_float4;

/* Field-for-field the layout of SimulationParams
 * (include/pbf/simulation_params.hpp:6-29). */
typedef struct pbf_params {
    float dt;
    float restDensity;
    float particleMass;
    float particleRadius;
    float collisionRestitution;
    float collisionFriction;
    float smoothingRadius;
    float lambdaEpsilon;
    int solverIterations;
    int substeps;
    pbf_float3 gravity;
    float scorrK;
    int scorrN;
    float scorrDeltaQ;
    float xsphViscosity;
    float vorticityStrength;
} pbf_params;

/* Collider layouts of include/pbf/colliders.hpp:8-24. */
typedef struct pbf_sphere { pbf_float3 center; float radius; } pbf_sphere;
typedef struct pbf_box { pbf_float3 center; pbf_float3 halfExtents; } pbf_box;
typedef struct pbf_plane { pbf_float3 point; pbf_float3 normal; } pbf_plane;

typedef struct pbf_solver pbf_solver;

/* ---- solver lifetime ----------------------------------------------------
 * Replaces PBFSolver's constructor/destructor.  create selects CUDA device
 * `device` (-1 = the current device). */
pbf_status pbf_solver_create(pbf_solver** out, int device);
void pbf_solver_destroy(pbf_solver* s);
/* Message of the last failed call on this handle ("" when none). */
const char* pbf_last_error(const pbf_solver* s);
/* Message of the last failed call that had no handle (create, stage calls). */
const char* pbf_global_last_error(void);

/* PBFSolver::initialize (src/pbf/pbf_solver.cu:23-116): validation, grid with
 * cell size = smoothingRadius, container = grid bounds, capacity, and the
 * neighbour capacity kMaxNeighbors = 256 (src/pbf/pbf_solver.cu:12). */
pbf_status pbf_initialize(pbf_solver* s, size_t max_particles, pbf_float3 min_bounds,
                          pbf_float3 max_bounds, const pbf_params* params);
/* Same with an explicit neighbour capacity (the reference hard-codes 256). */
pbf_status pbf_initialize_ex(pbf_solver* s, size_t max_particles, pbf_float3 min_bounds,
                             pbf_float3 max_bounds, const pbf_params* params,
                             int max_neighbors);

/* Same with compact neighbour lists: each rebuild counts every particle's
 * neighbours, scans the counts and stores each list contiguously, list_capacity
 * entries in all (memory follows the actual neighbour count instead of
 * max_particles x max_neighbors).  Results equal those of the slot-major lists
 * bit for bit.  A step whose lists need more than list_capacity entries fails
 * with PBF_ERR_OVERFLOW; max_neighbors still bounds each particle's count as in
 * the reference.  list_capacity must be in [1, 2^32 - 1]. */
pbf_status pbf_initialize_compact(pbf_solver* s, size_t max_particles, pbf_float3 min_bounds,
                                  pbf_float3 max_bounds, const pbf_params* params,
                                  int max_neighbors, size_t list_capacity);

/* PBFSolver::setParticles (src/pbf/pbf_solver.cu:118-152): host arrays,
 * finiteness checked, stable ids reset to the given order. */
pbf_status pbf_set_particles(pbf_solver* s, const pbf_float4* positions,
                             const pbf_float4* velocities, size_t count);
/* Same from device pointers (float4 arrays already resident in HBM). */
pbf_status pbf_set_particles_device(pbf_solver* s, const pbf_float4* d_positions,
                                    const pbf_float4* d_velocities, size_t count);

/* PBFSolver::setSpheres/setBoxes/setPlanes -> CollisionSystem setters
 * (src/pbf/collision_system.cu:53-131); count 0 clears. */
pbf_status pbf_set_spheres(pbf_solver* s, const pbf_sphere* spheres, size_t count);
pbf_status pbf_set_boxes(pbf_solver* s, const pbf_box* boxes, size_t count);
pbf_status pbf_set_planes(pbf_solver* s, const pbf_plane* planes, size_t count);

/* PBFSolver::step (src/pbf/pbf_solver.cu:186-328): one frame of
 * params.substeps substeps; synchronous. */
pbf_status pbf_step(pbf_solver* s);
/* PBFSolver::run() / run(frameCount) (src/pbf/pbf_solver.cu:330-343).  The
 * frames are launched back to back and checked once at the end; a failing
 * frame stops every later kernel, so the error is the first one. */
pbf_status pbf_run(pbf_solver* s, size_t frames);

/* PBFSolver::copyPositionsToHost / copyVelocitiesToHost
 * (src/pbf/pbf_solver.cu:345-379): API order, count must equal the active
 * count. */
pbf_status pbf_copy_positions(pbf_solver* s, pbf_float4* positions, size_t count);
pbf_status pbf_copy_velocities(pbf_solver* s, pbf_float4* velocities, size_t count);
/* Same into device memory. */
pbf_status pbf_copy_positions_device(pbf_solver* s, pbf_float4* d_positions, size_t count);
pbf_status pbf_copy_velocities_device(pbf_solver* s, pbf_float4* d_velocities, size_t count);

size_t pbf_particle_count(const pbf_solver* s);

/* ---- batched scenes (no counterpart in the reference) -------------------
 * Many independent scenes stepped together: one launch per stage for all of
 * them.  Each scene has its own particle count, container (== grid bounds,
 * cell size = smoothingRadius) and rest density, particle mass and XSPH
 * strength; every other field of `common` is shared.  XSPH must be on in
 * every scene or in none.  Cell keys are offset per scene, so one stable
 * sort orders all scenes and each scene's arithmetic is exactly that of a
 * solver initialised with that scene alone.  The handle then takes
 * pbf_set_particles with all scenes' particles concatenated in scene order
 * (the sum of the counts, no fewer), and pbf_step / pbf_run / pbf_copy_*
 * work on the concatenation.  Colliders set on the handle apply to every
 * scene in its own coordinates.  pbf_initialize returns the handle to one
 * scene. */
typedef struct pbf_scene {
    size_t count;
    pbf_float3 minBounds;
    pbf_float3 maxBounds;
    float restDensity;
    float particleMass;
    float xsphViscosity;
} pbf_scene;
pbf_status pbf_batch_initialize(pbf_solver* s, const pbf_scene* scenes, int scene_count,
                                const pbf_params* common, int max_neighbors);
/* Scenes of a batched handle (0 after pbf_initialize). */
int pbf_batch_scene_count(const pbf_solver* s);

/* Autotuner (no counterpart in the reference): for the six neighbour
 * kernels (walk + lambda, delta p, final walk, XSPH, vorticity,
 * confinement), times each at 64, 128, 256 and 512 threads per block in profiled
 * frames (`frames_per_trial` per size, after two untimed frames) and keeps
 * the fastest; then the radix sort's tile, 1,024 or 4,096 keys, timed on the
 * sort stage.  Results do not change (neither changes any arithmetic or the
 * sort's result); the particle state is restored, so tuning does not advance
 * the simulation.  Needs particles set. */
pbf_status pbf_autotune(pbf_solver* s, int frames_per_trial);
/* The block sizes in use, in the order above (count <= 6 entries). */
pbf_status pbf_block_sizes(const pbf_solver* s, int* sizes, int count);
/* Keys per radix-sort tile in use: 1,024 or 4,096 (chosen by the autotuner,
 * else 1,024 below 2^19 particles and 4,096 from there on). */
pbf_status pbf_sort_tile(const pbf_solver* s, int* keys_per_tile);
/* Lanes per particle of the list-writing walks in use: the value set by
 * pbf_set_walk_lanes, else 8 up to 20,480 particles, 4 below 32,768 and 1 from
 * there on (always 1 with compact lists; at most max_neighbors). */
pbf_status pbf_walk_lanes(const pbf_solver* s, int* lanes);
/* Sets the lanes per particle of the walks: 1, 2, 4 or 8, or 0 for the
 * default by scene size.  Results do not change.  A lane group pays when one small
 * scene leaves the GPU idle; many small solvers running at once on separate
 * streams fill it already and step faster with 1. */
pbf_status pbf_set_walk_lanes(pbf_solver* s, int lanes);

/* ---- reverse-mode derivative (no counterpart in the reference) ---------
 * Gradients of a loss on the final state of `steps` steps with respect to
 * the initial positions and velocities, restDensity (mass held fixed) and
 * xsphViscosity.  The differentiated step is integration, the density
 * constraint iterations with s_corr and the collision projection, the velocity
 * update, XSPH, vorticity confinement and the velocity response,
 * over neighbour lists
 * recorded by the forward (integer data, not differentiated).  The forward
 * runs the solver's own kernels: with one substep, one step from a state in
 * particle-id order is bit for bit pbf_step on that state; every substep
 * returns to particle-id order, so forward(x, v, a + b) equals
 * forward(forward(x, v, a), b).  A step of S substeps is taped as S substeps
 * of dt / S (checkpoint_every counts steps).  Sphere, box and plane colliders
 * (pbf_adjoint_set_*) are differentiated through replays of the projection
 * and the contact response.  The forward keeps (x, v) every `checkpoint_every` steps and
 * records its last segment; the backward recomputes each earlier segment
 * from its checkpoint.  State and gradient pointers may be host or device
 * memory.  Gradient arrays are float4 with w ignored. */
typedef struct pbf_adjoint pbf_adjoint;
pbf_status pbf_adjoint_create(pbf_adjoint** out, int device);
void pbf_adjoint_destroy(pbf_adjoint* a);
const char* pbf_adjoint_last_error(const pbf_adjoint* a);
pbf_status pbf_adjoint_initialize(pbf_adjoint* a, size_t count, pbf_float3 min_bounds,
                                  pbf_float3 max_bounds, const pbf_params* params,
                                  int max_neighbors, int checkpoint_every);
/* Replace restDensity and xsphViscosity (drops the recorded forward). */
pbf_status pbf_adjoint_set_physics(pbf_adjoint* a, float rest_density, float xsph_viscosity);
/* Colliders of the differentiated step, validated like pbf_set_spheres /
 * _boxes / _planes (count 0 clears; drops the recorded forward). */
pbf_status pbf_adjoint_set_spheres(pbf_adjoint* a, const pbf_sphere* spheres, size_t count);
pbf_status pbf_adjoint_set_boxes(pbf_adjoint* a, const pbf_box* boxes, size_t count);
pbf_status pbf_adjoint_set_planes(pbf_adjoint* a, const pbf_plane* planes, size_t count);
pbf_status pbf_adjoint_forward(pbf_adjoint* a, const pbf_float4* x0, const pbf_float4* v0,
                               int steps, pbf_float4* x_out, pbf_float4* v_out);
/* grad_x / grad_v: dL/dx, dL/dv of the last forward's final state;
 * returns dL/dx0, dL/dv0 and the two parameter derivatives. */
pbf_status pbf_adjoint_backward(pbf_adjoint* a, const pbf_float4* grad_x, const pbf_float4* grad_v,
                                pbf_float4* grad_x0, pbf_float4* grad_v0,
                                double* grad_rest_density, double* grad_xsph);

/* ---- streams, timing, diagnostics (no counterpart in the reference) ----- */
/* Run subsequent work on `stream` (a cudaStream_t); NULL restores the solver's
 * own stream.  The solver still synchronises its own calls. */
pbf_status pbf_set_stream(pbf_solver* s, void* stream);
/* Launch `frames` frames without synchronising; returns immediately. */
pbf_status pbf_run_async(pbf_solver* s, size_t frames);
/* Wait for queued work and report the device status of that work. */
pbf_status pbf_synchronize(pbf_solver* s);
/* Time `frames` frames with CUDA events on the solver's stream. */
pbf_status pbf_time_frames(pbf_solver* s, size_t frames, float* milliseconds);
/* Kernel launches one frame enqueues (graph nodes that run kernels). */
pbf_status pbf_kernels_per_frame(pbf_solver* s, int* kernels);
/* Runs one frame with CUDA events between its stages (a second captured
 * graph) and returns per-stage device milliseconds and launch counts, indexed
 * by stage id 0 .. pbf_stage_count()-1; the frame advances the simulation. */
pbf_status pbf_profile_frame(pbf_solver* s, float* stage_milliseconds, int* stage_launches);
int pbf_stage_count(void);
const char* pbf_stage_name(int stage);
/* Mean and max |rho/rho0 - 1| over the current particles and the neighbour
 * lists of the last rebuild (rho is computed but never exposed by the
 * reference, src/pbf/pbf_solver_kernels.cu:50-75). */
pbf_status pbf_density_error(pbf_solver* s, double* mean_error, double* max_error);
/* Working-order snapshot: positions, stable ids and neighbour counts in the
 * solver's current spatial order (any pointer may be NULL). */
pbf_status pbf_copy_working_state(pbf_solver* s, pbf_float4* positions, uint32_t* ids,
                                  int* neighbor_counts, size_t count);

/* ---- stage entry points (host arrays in and out) --------------------------
 * The reference's tests drive its kernels one by one; these mirror those
 * kernels with the same arguments, run the corresponding device code of this
 * library and copy the results back. */

/* SpatialGrid::initialize dims + SpatialGrid::build
 * (src/pbf/spatial_grid.cu:10-97, :139-226): stable sort of the given order
 * by cell key, cell_start/cell_end with -1 for empty cells (num_cells =
 * dims[0]*dims[1]*dims[2] entries each). */
pbf_status pbf_grid_dims(pbf_float3 min_bounds, pbf_float3 max_bounds, float cell_size,
                         int dims[3]);
pbf_status pbf_grid_build(const pbf_float4* positions, size_t count, pbf_float3 min_bounds,
                          pbf_float3 max_bounds, float cell_size, uint32_t* sorted_keys,
                          uint32_t* sorted_indices, int* cell_start, int* cell_end);

/* findNeighbors (src/pbf/neighbors.cu:3-91) over positions already in grid
 * order: slot-major lists neighbors[slot*stride + i]; overflow set to 1 when
 * any count exceeds max_neighbors. */
pbf_status pbf_find_neighbors(const pbf_float4* sorted_positions, size_t count,
                              const int* cell_start, const int* cell_end, const int dims[3],
                              pbf_float3 min_bounds, float cell_size, float smoothing_radius,
                              uint32_t* neighbors, int* neighbor_counts, int max_neighbors,
                              size_t stride, int* overflow);

/* computeLambda / computeDeltaPosition (src/pbf/pbf_solver_kernels.cu:26-182). */
pbf_status pbf_compute_lambda(const pbf_float4* positions, const uint32_t* neighbors,
                              const int* neighbor_counts, int max_neighbors, size_t count,
                              size_t stride, float smoothing_radius, float mass,
                              float rest_density, float epsilon, float* lambdas);
pbf_status pbf_compute_delta(const pbf_float4* positions, const uint32_t* neighbors,
                             const int* neighbor_counts, int max_neighbors,
                             const float* lambdas, size_t count, size_t stride,
                             float smoothing_radius, float mass, float rest_density,
                             float scorr_k, int scorr_n, float scorr_dq, pbf_float4* deltas);

/* applyXsphViscosity / computeVorticity / applyVorticityConfinement
 * (src/pbf/pbf_solver_kernels.cu:213-385). */
pbf_status pbf_xsph(const pbf_float4* positions, const uint32_t* neighbors,
                    const int* neighbor_counts, int max_neighbors, const pbf_float4* velocities,
                    pbf_float4* out_velocities, size_t count, size_t stride,
                    float smoothing_radius, float viscosity);
pbf_status pbf_vorticity(const pbf_float4* positions, const pbf_float4* velocities,
                         const uint32_t* neighbors, const int* neighbor_counts,
                         int max_neighbors, size_t count, size_t stride,
                         float smoothing_radius, pbf_float4* omega);
pbf_status pbf_confinement(const pbf_float4* positions, const uint32_t* neighbors,
                           const int* neighbor_counts, int max_neighbors,
                           const pbf_float4* omega, const pbf_float4* velocities,
                           pbf_float4* out_velocities, size_t count, size_t stride,
                           float smoothing_radius, float dt, float strength);

/* CollisionSystem::solve (src/pbf/collision_system.cu:133-172) in place;
 * PBF_ERR_RUNTIME when 32 passes do not converge.  pbf_collision_pass runs a
 * single projection kernel (kind 0 container, 1 spheres, 2 boxes, 3 planes,
 * src/pbf/collision_kernels.cu:47-234) and reports whether it corrected. */
pbf_status pbf_collide(pbf_float4* positions, size_t count, pbf_float3 container_min,
                       pbf_float3 container_max, const pbf_sphere* spheres, size_t sphere_count,
                       const pbf_box* boxes, size_t box_count, const pbf_plane* planes,
                       size_t plane_count, float particle_radius);
pbf_status pbf_collision_pass(pbf_float4* positions, size_t count, int kind,
                              pbf_float3 container_min, pbf_float3 container_max,
                              const pbf_sphere* spheres, size_t sphere_count,
                              const pbf_box* boxes, size_t box_count, const pbf_plane* planes,
                              size_t plane_count, float particle_radius, int* corrected);
/* CollisionSystem::resolveVelocities (src/pbf/collision_system.cu:182-218). */
pbf_status pbf_resolve_velocities(const pbf_float4* positions,
                                  const pbf_float4* incoming_velocities,
                                  pbf_float4* velocities, size_t count,
                                  pbf_float3 container_min, pbf_float3 container_max,
                                  const pbf_sphere* spheres, size_t sphere_count,
                                  const pbf_box* boxes, size_t box_count,
                                  const pbf_plane* planes, size_t plane_count,
                                  float particle_radius, float restitution, float friction);

/* Grid build that allocates no device memory.  No counterpart in the
 * reference: it is for callers that must not allocate while they run --
 * latency-bound or real-time loops, where cudaMalloc/cudaFree can block or
 * synchronise the whole device, and programs whose device memory belongs to a
 * pool or framework allocator that does not allow raw cudaMalloc beside it.
 * Same results as pbf_grid_build, but every array is a caller-owned DEVICE
 * array (num_cells = dims product entries for cell_start/cell_end) and the
 * work is enqueued on `stream` (a cudaStream_t, NULL = default stream)
 * without waiting for it.  Its working memory is one fixed array inside the
 * library, pbf_static_scratch_capacity() particles large (262,144), which every
 * GPU that loads the library keeps until the process exits; larger counts are
 * rejected with PBF_ERR_LENGTH before any other argument is checked.  The
 * first call on a device looks up that array's device address (make it before
 * any stream capture); the address is kept for the process, so the entry
 * point must not be used on a device after cudaDeviceReset of that device.
 * All calls share the array: calls whose GPU work overlaps in time race and
 * must be ordered by the caller (for example by issuing them on one
 * stream). */
pbf_status pbf_grid_build_static_scratch(const pbf_float4* d_positions, size_t count,
                                         pbf_float3 min_bounds, pbf_float3 max_bounds,
                                         float cell_size, uint32_t* d_sorted_keys,
                                         uint32_t* d_sorted_indices, int* d_cell_start,
                                         int* d_cell_end, void* stream);
size_t pbf_static_scratch_capacity(void);

/* integrate (src/pbf/integration.cu:6-32) in place on host arrays. */
pbf_status pbf_integrate(const pbf_float4* positions, pbf_float4* predicted,
                         pbf_float4* velocities, size_t count, float dt, pbf_float3 gravity);

/* Library version string. */
const char* pbf_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PBF103_H */
