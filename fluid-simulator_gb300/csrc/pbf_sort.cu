// pbf_sort.cu -- stable LSD radix sort of (cell key, index) pairs.
//
// Replaces cub::DeviceRadixSort::SortPairs over all 32 key bits
// (src/pbf/spatial_grid.cu:188-196).  A stable sort has one result whatever
// the digit schedule, so only the bits that can be non-zero are sorted:
// keys are clamped cell ids < num_cells.  Each pass is reduce-then-scan:
//   upsweep   per-tile digit histogram (shared-memory atomics) + digit totals
//   scan      one block per digit: exclusive scan over tiles + digit base
//   downsweep stable in-tile ranks (warp match + per-warp running counters,
//             items visited in index order) and scatter
// No kernel waits on another block, so nothing can spin.
#include "pbf_kernels.cuh"

#include <algorithm>

namespace pbf {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;                         // per thread
constexpr int kTile = kSortThreads * kSortItems;       // 4096 keys per tile
constexpr int kWarpChunk = kTile / kSortWarps;         // 512 consecutive keys per warp
constexpr int kMaxBins = 256;

__device__ __forceinline__ bool fatal(const unsigned* status) {
    return status != nullptr && (__ldcg(status) & kStatusFatalMask) != 0u;
}

__global__ void __launch_bounds__(kSortThreads)
k_upsweep(const uint32_t* __restrict__ keys, int n, int shift, uint32_t mask, int tiles,
          uint32_t* __restrict__ hist, uint32_t* __restrict__ totals,
          const unsigned* __restrict__ status) {
    if (fatal(status)) return;
    __shared__ uint32_t cnt[kMaxBins];
    const int bins = static_cast<int>(mask) + 1;
    for (int d = threadIdx.x; d < bins; d += kSortThreads) cnt[d] = 0;
    __syncthreads();
    const int base = blockIdx.x * kTile;
    const int end = min(n, base + kTile);
    for (int i = base + threadIdx.x; i < end; i += kSortThreads)
        atomicAdd(&cnt[(keys[i] >> shift) & mask], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < bins; d += kSortThreads) {
        const uint32_t c = cnt[d];
        hist[static_cast<size_t>(d) * tiles + blockIdx.x] = c;
        if (c) atomicAdd(&totals[d], c);
    }
}

// Block-wide exclusive scan helper over kSortThreads values.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* smem_warp,
                                                         uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) smem_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kSortWarps ? smem_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < kSortWarps) smem_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const uint32_t warp_base = warp ? smem_warp[warp - 1] : 0u;
    total = smem_warp[kSortWarps - 1];
    __syncthreads();
    return warp_base + incl - v;
}

// One block per digit: offsets[d][t] = base(d) + sum_{t' < t} hist[d][t'].
__global__ void __launch_bounds__(kSortThreads)
k_scan(uint32_t* __restrict__ hist, const uint32_t* __restrict__ totals, int tiles,
       const unsigned* __restrict__ status) {
    if (fatal(status)) return;
    __shared__ uint32_t warp_sums[kSortWarps];
    const int d = blockIdx.x;
    // Digit base: sum of the totals of all smaller digits.
    uint32_t part = 0;
    for (int e = threadIdx.x; e < d; e += kSortThreads) part += totals[e];
    uint32_t base_total;
    (void)block_exclusive_scan(part, warp_sums, base_total);
    uint32_t running = base_total;
    uint32_t* row = hist + static_cast<size_t>(d) * tiles;
    for (int t0 = 0; t0 < tiles; t0 += kSortThreads) {
        const int t = t0 + threadIdx.x;
        const uint32_t v = t < tiles ? row[t] : 0u;
        uint32_t chunk_total;
        const uint32_t ex = block_exclusive_scan(v, warp_sums, chunk_total);
        if (t < tiles) row[t] = running + ex;
        running += chunk_total;
    }
}

__global__ void __launch_bounds__(kSortThreads)
k_downsweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
            uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n, int shift,
            uint32_t mask, int tiles, const uint32_t* __restrict__ offsets,
            const unsigned* __restrict__ status) {
    if (fatal(status)) return;
    __shared__ uint32_t wcnt[kSortWarps][kMaxBins];
    __shared__ uint32_t tile_off[kMaxBins];
    const int bins = static_cast<int>(mask) + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < bins; d += kSortThreads) {
        tile_off[d] = offsets[static_cast<size_t>(d) * tiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) wcnt[w][d] = 0;
    }
    __syncthreads();

    const uint32_t lt_mask = (1u << lane) - 1u;
    const int base = blockIdx.x * kTile + warp * kWarpChunk;
    uint32_t k_reg[kSortItems], v_reg[kSortItems], r_reg[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        uint32_t key = 0, val = 0, digit = 0xffffffffu;
        if (valid) {
            key = keys_in[idx];
            val = vals_in ? vals_in[idx] : static_cast<uint32_t>(idx);
            digit = (key >> shift) & mask;
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const int leader = __ffs(peers) - 1;
        uint32_t prior = 0;
        if (valid && lane == leader) {
            prior = wcnt[warp][digit];
            wcnt[warp][digit] = prior + __popc(peers);
        }
        prior = __shfl_sync(0xffffffffu, prior, leader);
        k_reg[r] = key;
        v_reg[r] = val;
        r_reg[r] = valid ? prior + __popc(peers & lt_mask) : 0xffffffffu;
        __syncwarp();
    }
    __syncthreads();
    // Exclusive scan over the warps of each digit: earlier warps hold earlier keys.
    for (int d = threadIdx.x; d < bins; d += kSortThreads) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        if (r_reg[r] == 0xffffffffu) continue;
        const uint32_t digit = (k_reg[r] >> shift) & mask;
        const uint32_t dst = tile_off[digit] + wcnt[warp][digit] + r_reg[r];
        keys_out[dst] = k_reg[r];
        vals_out[dst] = v_reg[r];
    }
}

}  // namespace

SortPlan make_sort_plan(int n, uint64_t num_cells) {
    SortPlan p;
    p.n = n;
    p.tiles = std::max(1, (n + kTile - 1) / kTile);
    int bits = 1;
    while (bits < 32 && (uint64_t(1) << bits) < num_cells) ++bits;
    p.passes = (bits + 7) / 8;
    p.bits_per_pass = (bits + p.passes - 1) / p.passes;
    p.bins = 1 << p.bits_per_pass;
    return p;
}

size_t sort_scratch_bytes(int max_n) {
    const size_t tiles = std::max(1, (max_n + kTile - 1) / kTile);
    return (tiles * kMaxBins + kMaxBins) * sizeof(uint32_t);
}

int sort_kernel_count(const SortPlan& plan) { return plan.passes * 3; }

void launch_sort(const SortPlan& plan, const uint32_t* keys, uint32_t* sorted_keys,
                 uint32_t* sorted_idx, uint32_t* alt_keys, uint32_t* alt_idx, void* scratch,
                 const unsigned* status, cudaStream_t st) {
    uint32_t* hist = static_cast<uint32_t*>(scratch);
    uint32_t* totals = hist + static_cast<size_t>(plan.tiles) * kMaxBins;
    const uint32_t mask = static_cast<uint32_t>(plan.bins - 1);
    const uint32_t* kin = keys;
    const uint32_t* vin = nullptr;  // identity values on the first pass
    for (int p = 0; p < plan.passes; ++p) {
        // The last pass must land in sorted_*: alternate backwards from it.
        const bool to_sorted = ((plan.passes - 1 - p) % 2) == 0;
        uint32_t* kout = to_sorted ? sorted_keys : alt_keys;
        uint32_t* vout = to_sorted ? sorted_idx : alt_idx;
        const int shift = p * plan.bits_per_pass;
        cudaMemsetAsync(totals, 0, kMaxBins * sizeof(uint32_t), st);
        k_upsweep<<<plan.tiles, kSortThreads, 0, st>>>(kin, plan.n, shift, mask, plan.tiles, hist,
                                                       totals, status);
        k_scan<<<plan.bins, kSortThreads, 0, st>>>(hist, totals, plan.tiles, status);
        k_downsweep<<<plan.tiles, kSortThreads, 0, st>>>(kin, vin, kout, vout, plan.n, shift, mask,
                                                         plan.tiles, hist, status);
        kin = kout;
        vin = vout;
    }
}

}  // namespace pbf
