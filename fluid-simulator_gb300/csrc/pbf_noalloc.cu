// pbf_noalloc.cu -- a spatial-grid build that never allocates device memory.
//
// Some callers must not allocate GPU memory while they run: latency-bound or
// real-time loops, where cudaMalloc/cudaFree can block or synchronise the
// whole device, and host programs whose device memory belongs to a pool or a
// framework allocator that does not allow raw cudaMalloc next to it.  For
// them, pbf_grid_build_static_scratch runs the same hash + stable radix sort
// + cell-range kernels as the rest of the library, on device buffers the
// caller owns, and keeps its working memory (unsorted keys, the sort's
// ping-pong buffers, tile histograms and digit totals) in one fixed-size
// array that is part of the loaded library.
#include "pbf_common.h"
#include "pbf_kernels.cuh"

#include <cmath>
#include <limits>
#include <mutex>

namespace pbf {
namespace {

// Largest particle count the fixed scratch array serves.
constexpr size_t kStaticScratchParticles = size_t(1) << 18;  // 262,144
constexpr size_t kKeysBytes = kStaticScratchParticles * sizeof(uint32_t);

// Sort scratch (tile histograms + digit totals) for the capacity above,
// rounded up to the array's alignment.
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kSortBytes = align256(
    ((kStaticScratchParticles + kSortMinTile - 1) / kSortMinTile + 1) * kSortMaxBins * 4);
constexpr size_t kScratchBytes = 3 * kKeysBytes + kSortBytes;  // about 3.4 MB

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

// Host code cannot use g_static_scratch directly (on the host the name is a
// stand-in, not a device address), so its device address is looked up once
// per device, with that device current, and cached.  A cudaDeviceReset
// unloads the library's device code with the array, after which the cached
// address is stale: the entry point is not for use after a reset of its
// device in the same process.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

unsigned char* scratch_for_current_device() {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) fail(PBF_ERR_RUNTIME, "device index out of range");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cuda_check(cudaGetSymbolAddress(&p, g_static_scratch));
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    return g_scratch_ptr[dev];
}

}  // namespace
}  // namespace pbf

using namespace pbf;

extern "C" {

size_t pbf_static_scratch_capacity(void) { return kStaticScratchParticles; }

pbf_status pbf_grid_build_static_scratch(const pbf_float4* d_positions, size_t count,
                                         pbf_float3 min_bounds, pbf_float3 max_bounds,
                                         float cell_size, uint32_t* d_sorted_keys,
                                         uint32_t* d_sorted_indices, int* d_cell_start,
                                         int* d_cell_end, void* stream) {
    return guarded(nullptr, [&]() {
        if (count > kStaticScratchParticles)
            fail(PBF_ERR_LENGTH,
                 "particle count exceeds the static scratch capacity of 262144 particles");
        if (!std::isfinite(cell_size) || cell_size <= 0.0f)
            fail(PBF_ERR_INVALID_ARGUMENT, "cellSize must be greater than zero");
        const float lo[3] = {min_bounds.x, min_bounds.y, min_bounds.z};
        const float hi[3] = {max_bounds.x, max_bounds.y, max_bounds.z};
        int d[3];
        for (int a = 0; a < 3; ++a) {
            if (!std::isfinite(lo[a]) || !std::isfinite(hi[a]) || hi[a] <= lo[a])
                fail(PBF_ERR_INVALID_ARGUMENT, "Invalid spatial grid bounds");
            const double c = std::ceil((double(hi[a]) - double(lo[a])) / double(cell_size));
            if (!std::isfinite(c) || c < 1.0 || c > double(std::numeric_limits<int>::max()))
                fail(PBF_ERR_LENGTH, "Spatial grid axis exceeds integer capacity");
            d[a] = static_cast<int>(c);
        }
        const size_t maxCells = std::numeric_limits<uint32_t>::max();
        if (size_t(d[0]) > maxCells / size_t(d[1]) ||
            size_t(d[0]) * size_t(d[1]) > maxCells / size_t(d[2]))
            fail(PBF_ERR_LENGTH, "Spatial grid exceeds 32-bit key capacity");
        const size_t cells = size_t(d[0]) * size_t(d[1]) * size_t(d[2]);
        if (!d_cell_start || !d_cell_end)
            fail(PBF_ERR_INVALID_ARGUMENT, "cell_start and cell_end must not be null");
        if (count && (!d_positions || !d_sorted_keys || !d_sorted_indices))
            fail(PBF_ERR_INVALID_ARGUMENT, "device arrays must not be null");

        cudaStream_t st = static_cast<cudaStream_t>(stream);
        unsigned char* base = scratch_for_current_device();
        uint32_t* keys = reinterpret_cast<uint32_t*>(base);
        uint32_t* alt_keys = reinterpret_cast<uint32_t*>(base + kKeysBytes);
        uint32_t* alt_idx = reinterpret_cast<uint32_t*>(base + 2 * kKeysBytes);
        void* sort_scratch = base + 3 * kKeysBytes;

        // Empty cells read -1, like SpatialGrid::build (src/pbf/spatial_grid.cu:201-204).
        cuda_check(cudaMemsetAsync(d_cell_start, 0xff, cells * sizeof(int), st));
        cuda_check(cudaMemsetAsync(d_cell_end, 0xff, cells * sizeof(int), st));
        if (count == 0) return;
        const int n = static_cast<int>(count);
        GridConst g{};
        g.minx = lo[0];
        g.miny = lo[1];
        g.minz = lo[2];
        g.cell = cell_size;
        g.gx = d[0];
        g.gy = d[1];
        g.gz = d[2];
        launch_grid_keys(reinterpret_cast<const float4*>(d_positions), keys, n, g, st);
        // Nothing an earlier call left in the shared array is read: every
        // pass rewrites the tile histograms it reads (upsweep), the digit
        // totals are either rewritten by the scan launch or, with few tiles,
        // not read at all (the downsweep sums the histograms itself), and the
        // key buffers are written before they are read.
        const SortPlan plan = make_sort_plan(n, cells);
        launch_sort(plan, keys, d_sorted_keys, d_sorted_indices, alt_keys, alt_idx, sort_scratch,
                    nullptr, st);
        launch_cell_ranges(d_sorted_keys, d_cell_start, d_cell_end, n, nullptr, st);
        cuda_check(cudaGetLastError());
    });
}

}  // extern "C"
