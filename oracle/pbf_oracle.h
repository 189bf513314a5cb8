/*
 * pbf_oracle.h -- CPU oracle for the Position Based Fluids step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a CPU restatement of the reference
 * solver's step (DusanCojic/Fluid-Simulator, src/pbf/pbf_solver.cu:186-328)
 * used as the parity checker for the CUDA library and as the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline arm may load it; the product library never links it.
 *
 * Two arithmetic modes share one algorithm:
 *   - FP32 "mirror": integer work (cell hash, stable sort, cell ranges,
 *     neighbour lists) exactly as the reference; floating-point work with the
 *     same operation order and fused multiply-adds as the CUDA kernels of
 *     this repository, so CUDA-vs-oracle comparisons are bit-exact.
 *   - FP64: the reference's formulas evaluated in double precision, the
 *     accuracy yardstick for positions and velocities.
 */
#ifndef PBF_ORACLE_H
#define PBF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float x, y, z; } orc_float3;
typedef struct { float x, y, z, w; } orc_float4;

/* Same field order as SimulationParams (include/pbf/simulation_params.hpp:6-29). */
typedef struct {
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
    orc_float3 gravity;
    float scorrK;
    int scorrN;
    float scorrDeltaQ;
    float xsphViscosity;
    float vorticityStrength;
} orc_params;

typedef struct { orc_float3 center; float radius; } orc_sphere;
typedef struct { orc_float3 center; orc_float3 halfExtents; } orc_box;
typedef struct { orc_float3 point; orc_float3 normal; } orc_plane;
typedef struct { orc_float3 min; orc_float3 max; } orc_container;

enum {
    ORC_OK = 0,
    ORC_ERR_INVALID = 1,
    ORC_ERR_LENGTH = 2,
    ORC_ERR_OVERFLOW = 3,
    ORC_ERR_NOT_CONVERGED = 4
};

/* ---- spatial grid (src/pbf/spatial_grid.cu) ---------------------------- */
int orc_grid_dims(orc_float3 minB, orc_float3 maxB, float cell, int dims[3]);
uint32_t orc_cell_key(orc_float4 p, orc_float3 minB, float cell, const int dims[3]);
/* Stable sort by cell key of the current order; cellStart/cellEnd get -1 for
 * empty cells, as SpatialGrid::build. */
void orc_grid_build(const orc_float4* pos, size_t n, orc_float3 minB, float cell,
                    const int dims[3], uint32_t* sortedKeys, uint32_t* sortedIdx,
                    int* cellStart, int* cellEnd);

/* ---- neighbour search (src/pbf/neighbors.cu:3-91), slot-major output ----- */
int orc_find_neighbors(const orc_float4* sortedPos, size_t n, const int* cellStart,
                       const int* cellEnd, const int dims[3], orc_float3 minB,
                       float cell, float h, uint32_t* neighbors, int* counts,
                       int maxNeighbors, size_t stride);

/* ---- single-stage FP32 mirrors of the constraint / velocity kernels ------ */
void orc_lambda(const orc_float4* pos, const uint32_t* nbrs, const int* counts,
                int maxNeighbors, size_t n, size_t stride, float h, float mass,
                float rho0, float eps, float* lambda);
void orc_delta(const orc_float4* pos, const uint32_t* nbrs, const int* counts,
               int maxNeighbors, const float* lambda, size_t n, size_t stride,
               float h, float mass, float rho0, float k, int nexp, float dq,
               orc_float4* delta);
float orc_scorr(float d2, float h, float k, int nexp, float dq);
float orc_poly6(float d2, float h);
void orc_spiky(float dx, float dy, float dz, float h, float out[3]);
void orc_xsph(const orc_float4* pos, const uint32_t* nbrs, const int* counts,
              int maxNeighbors, const orc_float4* vin, orc_float4* vout, size_t n,
              size_t stride, float h, float c);
void orc_vorticity(const orc_float4* pos, const orc_float4* vel, const uint32_t* nbrs,
                   const int* counts, int maxNeighbors, size_t n, size_t stride,
                   float h, orc_float4* omega);
void orc_confinement(const orc_float4* pos, const uint32_t* nbrs, const int* counts,
                     int maxNeighbors, const orc_float4* omega, const orc_float4* vin,
                     orc_float4* vout, size_t n, size_t stride, float h, float dt,
                     float eps);

/* ---- collisions (src/pbf/collision_kernels.cu) -------------------------- */
/* One pass of each projection kernel; returns 1 when any particle was marked. */
int orc_solve_container(orc_float4* pos, size_t n, orc_container c, float r);
int orc_solve_spheres(orc_float4* pos, size_t n, const orc_sphere* s, size_t ns, float r);
int orc_solve_boxes(orc_float4* pos, size_t n, const orc_box* b, size_t nb, float r);
int orc_solve_planes(orc_float4* pos, size_t n, const orc_plane* p, size_t np, float r);
/* CollisionSystem::solve: up to maxPasses passes; ORC_ERR_NOT_CONVERGED else OK. */
int orc_collide(orc_float4* pos, size_t n, orc_container c, const orc_sphere* s,
                size_t ns, const orc_box* b, size_t nb, const orc_plane* p, size_t np,
                float r, int maxPasses);
void orc_resolve_velocities(const orc_float4* pos, const orc_float4* vin, orc_float4* vel,
                            size_t n, orc_container c, const orc_sphere* s, size_t ns,
                            const orc_box* b, size_t nb, const orc_plane* p, size_t np,
                            float r, float restitution, float friction);

/* ---- whole solver (PBFSolver) ------------------------------------------- */
typedef struct orc_solver orc_solver;
/* precision: 32 (FP32 mirror) or 64 (FP64 reference formulas). */
orc_solver* orc_solver_create(int precision);
void orc_solver_destroy(orc_solver* s);
void orc_solver_set_threads(orc_solver* s, int threads);
int orc_solver_initialize(orc_solver* s, size_t maxParticles, orc_float3 minB,
                          orc_float3 maxB, const orc_params* params, int maxNeighbors);
int orc_solver_set_particles(orc_solver* s, const orc_float4* pos, const orc_float4* vel,
                             size_t n);
int orc_solver_set_colliders(orc_solver* s, const orc_sphere* sp, size_t ns,
                             const orc_box* bx, size_t nb, const orc_plane* pl, size_t np);
int orc_solver_step(orc_solver* s);
/* Positions / velocities in the API (stable id) order, as float. */
int orc_solver_copy_positions(const orc_solver* s, orc_float4* out, size_t n);
int orc_solver_copy_velocities(const orc_solver* s, orc_float4* out, size_t n);
/* Working-order state: positions, stable ids and the last neighbour lists. */
int orc_solver_copy_working(const orc_solver* s, orc_float4* pos, uint32_t* ids,
                            int* counts, size_t n);
/* Mean and max |rho/rho0 - 1| over the current working order and lists. */
int orc_solver_density_error(const orc_solver* s, double* meanErr, double* maxErr);

/* Density error of a set of positions, evaluated the same way whichever
 * solver produced them: rho_i = m * sum_j W(x_i - x_j) over every particle
 * within h (self included), poly6 in double over cells of size h; writes
 * mean and max |rho/rho0 - 1| and the fraction of particles above 10 %. */
int orc_density_stats(const orc_float4* pos, size_t n, orc_float3 minB, orc_float3 maxB,
                      float h, float mass, float rho0, double* meanErr, double* maxErr,
                      double* fracAbove10);

/* ---- FP64 forward-mode restatement of the differentiated step
 * (pbf_diff_oracle.cpp): `steps` steps of integration, the density
 * constraint with s_corr and the container clamp, velocity update, XSPH and
 * container contacts, from (x0, v0), with ntan <= 12 tangent directions:
 * tx0 / tv0 (ntan * n * 3 doubles or NULL) and trho / tc (ntan doubles or
 * NULL) seed d(x0), d(v0), d(restDensity), d(xsphViscosity).  With
 * `states` (steps * 2 * n float4: x then v at the start of each step, or
 * NULL) the values restart from that trajectory at every step while the
 * tangents carry on: the derivative linearised about a given (for instance
 * FP32) trajectory.  Outputs the final x, v (n * 3) and their tangents
 * (ntan * n * 3, may be NULL). */
int orc_diff_rollout(size_t n, const orc_float4* x0, const orc_float4* v0, const double* tx0,
                     const double* tv0, const double* trho, const double* tc, int ntan,
                     const orc_params* prm, orc_float3 lo, orc_float3 hi, int steps,
                     const orc_float4* states, double* x_out, double* v_out, double* tx_out,
                     double* tv_out);
/* Same, with restDensity and xsphViscosity taken from phys[0], phys[1] in
 * double instead of from params (phys may be NULL). */
int orc_diff_rollout_phys(size_t n, const orc_float4* x0, const orc_float4* v0, const double* tx0,
                          const double* tv0, const double* trho, const double* tc, int ntan,
                          const orc_params* prm, orc_float3 lo, orc_float3 hi, int steps,
                          const orc_float4* states, double* x_out, double* v_out, double* tx_out,
                          double* tv_out, const double* phys);
/* Same with sphere, box and plane colliders (projection and contact
 * response); ORC_ERR_NOT_CONVERGED when a projection does not converge. */
int orc_diff_rollout_col(size_t n, const orc_float4* x0, const orc_float4* v0, const double* tx0,
                         const double* tv0, const double* trho, const double* tc, int ntan,
                         const orc_params* prm, orc_float3 lo, orc_float3 hi, int steps,
                         const orc_float4* states, double* x_out, double* v_out, double* tx_out,
                         double* tv_out, const double* phys, const orc_sphere* sp, size_t ns,
                         const orc_box* bx, size_t nb, const orc_plane* pl, size_t np);

#ifdef __cplusplus
}
#endif

#endif
