// pbf_kernels.cuh -- kernel launchers of the PBF step (host-callable).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_collide.cuh"
#include "pbf_math.cuh"

namespace pbf {

// Per-scene constants of a batched solver: the scene's own grid (its cell
// keys are offset by cell_base, so one sort orders all scenes, scene by
// scene), its container and the density terms that vary between scenes.
struct SceneConst {
    GridConst g;
    uint32_t cell_base;
    float cminx, cminy, cminz, cmaxx, cmaxy, cmaxz;
    float rho0, mass, gs, gs2, xsph_c;
};

// Everything a step kernel needs, passed by value.
struct StepConst {
    KernelConst k;
    ScorrConst sc;
    GridConst g;
    Colliders col;
    float mass, rho0, lambda_eps, gs, gs2;  // gs = mass / rho0
    float dt, inv_dt;                        // substep dt and 1/dt (host float divide)
    float gravx, gravy, gravz;
    float particle_radius, restitution, friction;
    float xsph_c, vort_eps;
    int max_nb;
    size_t stride;  // slot stride of the neighbour lists
    // Batched solver: scene table and the scene of every particle slot
    // (scenes occupy fixed contiguous slot ranges); null for one scene.
    const SceneConst* scenes;
    const uint16_t* sid;
    // Threads per block of the tuned kernels (TunedKernel order); 0 = kBlock.
    int blk[6];
    // Compact neighbour lists: particle i's list is nbr[nb_off[i] + k] inside
    // nb_cap entries.  Null: slot-major lists, nbr[k * stride + i].
    const uint32_t* nb_off;
    size_t nb_cap;
    // Lanes per particle in the list-writing walks (1, 2 or 4; 0 = 1): more
    // than one splits each particle's stencil rows over a lane group, for
    // scenes too small to fill the GPU.  Slot-major lists only.
    int walk_lanes;
    // Leave out of the walks the stencil cells that cannot hold a neighbour
    // (their box is farther than h from the particle).  Needs cell tables
    // built from the walked positions themselves, as the step's rebuilds
    // are; off for the stage entry points, which take the caller's tables.
    bool prune_cells;
};

// Lanes per particle for the walks of an n-particle scene (slot-major lists
// with max_nb slots).
int default_walk_lanes(size_t n, int max_nb);

// Stride (floats) of the x, y, z component arrays the walks read, for n
// particles: a multiple of 64 (every array 256-byte aligned, so the walk's
// 16-byte loads are aligned) with at least kSoaTail readable floats past the
// last particle, because the walk tests candidates in 32-wide chunks that
// may run past the end of a cell row (those lanes are masked off).
constexpr size_t kSoaTail = 32;
constexpr size_t soa_stride_for(size_t n) { return (n + kSoaTail + 63) / 64 * 64; }

// Kernels whose block size the solver's autotuner chooses.
enum TunedKernel { kTunedSearchLambda, kTunedDelta, kTunedSearch, kTunedXsph, kTunedVorticity,
                   kTunedConfine, kTunedCount };
constexpr int kMaxTunedBlock = 512;

constexpr int kBlock = 256;

inline unsigned blocks_for(size_t n, int block = kBlock) {
    return static_cast<unsigned>((n + block - 1) / block);
}

// Launches kernel k on stream st; launch errors throw like cuda_check.
void launch_error_check(cudaError_t e);
template <typename... P, typename... A>
inline void launch_k(void (*k)(P...), unsigned grid, unsigned block, cudaStream_t st, A&&... a) {
    if (grid == 0) return;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cfg.attrs = nullptr;
    cfg.numAttrs = 0;
    launch_error_check(cudaLaunchKernelEx(&cfg, k, static_cast<P>(a)...));
}

// --- step kernels (pbf_kernels.cu) -----------------------------------------
void launch_predict(const float4* x, const float4* v, float4* xs, float4* vin, uint32_t* keys,
                    int n, const StepConst& c, const unsigned* status, cudaStream_t st);
void launch_cell_ranges(const uint32_t* skeys, int* cell_start, int* cell_end, int n,
                        const unsigned* status, cudaStream_t st);
// Reorders predicted positions (float4 and x/y/z component arrays for the
// search) and composes the substep permutation; org_out may be null.
void launch_gather_xs(const uint32_t* perm, const float4* xs_in, float4* xs_out,
                      const uint32_t* org_in, uint32_t* org_out, float* sx, float* sy, float* sz,
                      int n, const unsigned* status, cudaStream_t st);
// launch_gather_xs with org_out set, fused with the refresh of first[]
// (lower bound of every cell key, cells + 1 entries), which is updated in
// place: its previous contents only seed the search.
void launch_gather_first(const uint32_t* perm, const float4* xs_in, float4* xs_out,
                         const uint32_t* org_in, uint32_t* org_out, float* sx, float* sy, float* sz,
                         int n, const uint32_t* skeys, uint64_t cells, int* first,
                         const unsigned* status, cudaStream_t st);
void launch_search(const float4* xs, const float* sx, const float* sy, const float* sz,
                   const int* first, const StepConst& c, int n, uint32_t* nbr, int* cnt, float* lam,
                   unsigned* status, bool with_lambda, cudaStream_t st);
// The final walk with XSPH in a second pass over the new lists (v: updated
// velocities; resolve: apply the velocity response against vin as well).
void launch_search_xsph(const float4* xs, const float* sx, const float* sy, const float* sz,
                        const int* first, const StepConst& c, int n, uint32_t* nbr, int* cnt,
                        const float4* v, float4* v_out, const float4* vin, bool resolve,
                        unsigned* status, cudaStream_t st);
// moved (optional): per slot, bit a set where the collision projection
// changed component a of the position; pre (optional): the position before
// the projection.
void launch_delta_apply(const float4* xs, const uint32_t* nbr, const int* cnt, const float* lam,
                        const StepConst& c, int n, float4* xs_out, uint32_t* keys_out,
                        unsigned* status, cudaStream_t st, uint8_t* moved = nullptr,
                        float4* pre = nullptr);
// Compact lists: neighbour counts of the walk (no list written), then the
// exclusive scan of the counts into off (n + 1 entries; a total above cap
// sets kStatusListOverflow).  scratch: nb_scan_scratch_words(n) words.
void launch_count(const float4* xs, const float* sx, const float* sy, const float* sz,
                  const int* first, const StepConst& c, int n, int* cnt, unsigned* status,
                  cudaStream_t st);
size_t nb_scan_scratch_words(size_t n);
void launch_nb_scan(const int* cnt, uint32_t* off, size_t cap, int n, uint32_t* scratch,
                    unsigned* status, cudaStream_t st);
// id_new may be null (ids not carried).
void launch_finalize(const uint32_t* org, const float4* x_old, const float4* vin_old,
                     const float4* v_old, const uint32_t* id_old, const float4* xs, int n,
                     const StepConst& c, float4* v_new, float4* vin_new, uint32_t* id_new,
                     const unsigned* status, cudaStream_t st);
void launch_xsph(const float4* x, const float4* v, const uint32_t* nbr, const int* cnt,
                 const StepConst& c, int n, float4* v_out, const float4* vin, bool resolve,
                 const unsigned* status, cudaStream_t st);
// store_norm: w = |omega| (the form launch_confine reads) instead of 0.
void launch_vorticity(const float4* x, const float4* v, const uint32_t* nbr, const int* cnt,
                      const StepConst& c, int n, float4* omega, bool store_norm,
                      const unsigned* status, cudaStream_t st);
// Sets w = |omega| in a vorticity array written with w = 0.
void launch_omega_norm(float4* omega, int n, cudaStream_t st);
// omega: w = |omega| (launch_vorticity with store_norm, or launch_omega_norm).
void launch_confine(const float4* x, const uint32_t* nbr, const int* cnt, const float4* omega,
                    const float4* v, const StepConst& c, int n, float4* v_out,
                    const float4* vin, bool resolve, const unsigned* status, cudaStream_t st);
void launch_resolve(const float4* x, const float4* vin, float4* v, const StepConst& c, int n,
                    const unsigned* status, cudaStream_t st);
void launch_scatter_by_id(const float4* vals, const uint32_t* id, float4* out, int n,
                          cudaStream_t st);
void launch_iota(uint32_t* a, int n, cudaStream_t st);
void launch_density(const float4* x, const uint32_t* nbr, const int* cnt, const StepConst& c,
                    int n, float* err, cudaStream_t st);

// --- stage kernels for the standalone entry points -------------------------
void launch_grid_keys(const float4* pos, uint32_t* keys, int n, const GridConst& g,
                      cudaStream_t st);
void launch_lambda_list(const float4* xs, const uint32_t* nbr, const int* cnt,
                        const StepConst& c, int n, float* lam, cudaStream_t st);
void launch_delta_list(const float4* xs, const uint32_t* nbr, const int* cnt, const float* lam,
                       const StepConst& c, int n, float4* delta, cudaStream_t st);
void launch_collide(float4* pos, int n, const StepConst& c, int kind, unsigned* flag,
                    cudaStream_t st);
void launch_integrate(const float4* x, float4* xs, float4* v, int n, const StepConst& c,
                      cudaStream_t st);

// --- stable LSD radix sort of (key, index) pairs (pbf_sort.cu) ---------------
struct SortPlan {
    int n = 0;
    int tile = 0;  // keys per tile
    int tiles = 0;
    int passes = 0;
    int bits_per_pass = 0;
    int bins = 0;
};
// Smallest tile (keys) any plan uses, and the most digit bins of a pass:
// the scratch of n keys holds (ceil(n / kSortMinTile) + 1) * kSortMaxBins words.
constexpr int kSortMinTile = 1024;
constexpr int kSortMaxTile = 4096;
constexpr int kSortMaxBins = 256;
// tile: keys per tile, kSortMinTile or kSortMaxTile; anything else picks by
// size (the smaller tiles below 2^19 keys).  The result does not depend on it.
SortPlan make_sort_plan(int n, uint64_t num_cells, int tile = 0);
// Scratch bytes for hist/totals of a plan with up to n keys.
size_t sort_scratch_bytes(int max_n);
// Sorts keys (current order) into sorted_keys/sorted_idx; values start as the
// identity.  alt_keys/alt_idx are ping-pong buffers of n entries.
void launch_sort(const SortPlan& plan, const uint32_t* keys, uint32_t* sorted_keys,
                 uint32_t* sorted_idx, uint32_t* alt_keys, uint32_t* alt_idx, void* scratch,
                 const unsigned* status, cudaStream_t st);
// Number of kernel launches launch_sort issues.
int sort_kernel_count(const SortPlan& plan);

}  // namespace pbf
