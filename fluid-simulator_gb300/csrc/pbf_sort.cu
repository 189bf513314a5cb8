// pbf_sort.cu -- stable LSD radix sort of (cell key, index) pairs.
//
// Replaces cub::DeviceRadixSort::SortPairs over all 32 key bits
// (src/pbf/spatial_grid.cu:188-196).  A stable sort has one result whatever
// the digit schedule, so only the bits that can be non-zero are sorted:
// keys are clamped cell ids < num_cells.  Each pass is reduce-then-scan over
// tiles of 1,024 or 4,096 keys:
//   upsweep   per-tile digit histogram (shared-memory atomics)
//   scan      one block per digit: exclusive scan over tiles + digit total
//             (skipped up to kSumTilesMax tiles: the downsweep blocks then
//             sum the few tile histograms they need themselves)
//   downsweep digit bases from the totals, stable in-tile ranks (warp match
//             + per-warp running counters, items visited in index order),
//             tile staged in shared memory in digit order, then written out
//             as contiguous runs (coalesced stores)
// Up to 16,384 keys one thread-block cluster does every pass in a single
// launch (k_sort_cluster: the keys stay in the CTAs' shared memory and move
// between them through distributed shared memory, with cluster barriers).
// No kernel spins on another block: the cluster barrier is the hardware's,
// and every CTA of a cluster is resident together.
#include "pbf_kernels.cuh"

#include <cooperative_groups.h>

#include <algorithm>

namespace pbf {

namespace {

// Two tile shapes: 512 threads x 8 keys (4,096-key tiles) for large sorts,
// 256 threads x 4 keys (1,024-key tiles) below kSmallTileBelow keys, where
// 4,096-key tiles would leave most SMs idle (measured per sort: 22.0 against
// 24.6 us at 65,536 keys, 44.7 against 55.8 us at 1,048,576 for the larger
// tiles).  A stable sort has one result whatever the tiling.
constexpr int kMaxBins = kSortMaxBins;
template <int T, int ITEMS>
struct Shape {
    static constexpr int kThreads = T;
    static constexpr int kWarps = T / 32;
    static constexpr int kItems = ITEMS;                // per thread
    static constexpr int kTile = T * ITEMS;
    static constexpr int kWarpChunk = kTile / kWarps;   // consecutive keys per warp
    static_assert(kMaxBins <= T, "one digit per thread in the prologues");
};
using Large = Shape<512, 8>;
using Small = Shape<256, 4>;
static_assert(Small::kTile == kSortMinTile, "scratch is sized for the smallest tile");
constexpr int kSmallTileBelow = 1 << 19;
// Up to this many tiles the downsweep blocks sum the tile histograms
// themselves (at most kSumTilesMax loads per digit) instead of a scan launch.
// Measured per sort: 15.1 against 18.8 us at 16,384 keys (16 tiles); with 64
// tiles (65,536 keys) the sums cost more than the launch: 31.8 against 20.4 us.
constexpr int kSumTilesMax = 32;

__device__ __forceinline__ bool fatal(const unsigned* status) {
    return status != nullptr && (__ldcg(status) & kStatusFatalMask) != 0u;
}

template <class S>
__global__ void __launch_bounds__(S::kThreads)
k_upsweep(const uint32_t* __restrict__ keys, int n, int shift, uint32_t mask, int tiles,
          uint32_t* __restrict__ hist, const unsigned* __restrict__ status) {
    if (fatal(status)) return;
    __shared__ uint32_t cnt[kMaxBins];
    const int bins = static_cast<int>(mask) + 1;
    for (int d = threadIdx.x; d < bins; d += S::kThreads) cnt[d] = 0;
    __syncthreads();
    const int base = blockIdx.x * S::kTile;
    const int end = min(n, base + S::kTile);
    for (int i = base + threadIdx.x; i < end; i += S::kThreads)
        atomicAdd(&cnt[(keys[i] >> shift) & mask], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < bins; d += S::kThreads)
        hist[static_cast<size_t>(d) * tiles + blockIdx.x] = cnt[d];
}

// Block-wide exclusive scan over the block's values (one per thread).
template <int kSortWarps>
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

// One block per digit: hist[d][t] <- sum_{t' < t} hist[d][t'], totals[d] <- row sum.
template <class S>
__global__ void __launch_bounds__(S::kThreads)
k_scan(uint32_t* __restrict__ hist, uint32_t* __restrict__ totals, int tiles,
       const unsigned* __restrict__ status) {
    if (fatal(status)) return;
    __shared__ uint32_t warp_sums[S::kWarps];
    const int d = blockIdx.x;
    uint32_t running = 0;
    uint32_t* row = hist + static_cast<size_t>(d) * tiles;
    for (int t0 = 0; t0 < tiles; t0 += S::kThreads) {
        const int t = t0 + threadIdx.x;
        const uint32_t v = t < tiles ? row[t] : 0u;
        uint32_t chunk_total;
        const uint32_t ex = block_exclusive_scan<S::kWarps>(v, warp_sums, chunk_total);
        if (t < tiles) row[t] = running + ex;
        running += chunk_total;
    }
    if (threadIdx.x == 0) totals[d] = running;
}

template <class S>
__global__ void __launch_bounds__(S::kThreads)
k_downsweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
            uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n, int shift,
            uint32_t mask, int tiles, const uint32_t* __restrict__ offsets,
            const uint32_t* __restrict__ totals, const unsigned* __restrict__ status,
            bool sum_tiles) {
    if (fatal(status)) return;
    // The per-warp digit counters are dead once every item holds its
    // in-tile position, so the staging area for the tile reuses them.
    constexpr int kCountWords = S::kWarps * kMaxBins;
    constexpr int kStageWords = 2 * S::kTile;
    __shared__ uint32_t pool[kCountWords > kStageWords ? kCountWords : kStageWords];
    __shared__ uint32_t tile_off[kMaxBins];    // global start of each digit's run
    __shared__ uint32_t tile_start[kMaxBins];  // in-tile start of each digit
    __shared__ uint32_t warp_sums[S::kWarps];
    uint32_t(*wcnt)[kMaxBins] = reinterpret_cast<uint32_t(*)[kMaxBins]>(pool);
    uint32_t* skey = pool;
    uint32_t* sval = pool + S::kTile;

    const int bins = static_cast<int>(mask) + 1;
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int tile_base = blockIdx.x * S::kTile;
    const int base = tile_base + warp * S::kWarpChunk;
    uint32_t k_reg[S::kItems], v_reg[S::kItems], r_reg[S::kItems];
    // All loads of the warp's chunk are issued first; their latency overlaps
    // the prologue.
#pragma unroll
    for (int r = 0; r < S::kItems; ++r) {
        const int idx = base + r * 32 + lane;
        k_reg[r] = idx < n ? keys_in[idx] : 0u;
        v_reg[r] = idx < n ? (vals_in ? vals_in[idx] : static_cast<uint32_t>(idx)) : 0u;
    }
    for (int d = tid; d < bins; d += S::kThreads) {
#pragma unroll
        for (int w = 0; w < S::kWarps; ++w) wcnt[w][d] = 0;
    }
    // Digit bases: exclusive scan of the digit totals.  With sum_tiles (few
    // tiles, no scan launch) `offsets` holds the raw tile histograms: each
    // block sums its digit's row itself, all tiles for the total and the
    // tiles before its own for its offset.
    {
        uint32_t tot = 0u, before = 0u;
        if (tid < bins) {
            if (sum_tiles) {
                const uint32_t* row = offsets + static_cast<size_t>(tid) * tiles;
                for (int t = 0; t < tiles; ++t) {
                    const uint32_t v = row[t];
                    tot += v;
                    before += t < static_cast<int>(blockIdx.x) ? v : 0u;
                }
            } else {
                tot = totals[tid];
                before = offsets[static_cast<size_t>(tid) * tiles + blockIdx.x];
            }
        }
        uint32_t all;
        const uint32_t dbase = block_exclusive_scan<S::kWarps>(tot, warp_sums, all);
        if (tid < bins) tile_off[tid] = dbase + before;
    }
    __syncthreads();

    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < S::kItems; ++r) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        const uint32_t key = k_reg[r];
        const uint32_t digit = valid ? (key >> shift) & mask : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const int leader = __ffs(peers) - 1;
        uint32_t prior = 0;
        if (valid && lane == leader) {
            prior = wcnt[warp][digit];
            wcnt[warp][digit] = prior + __popc(peers);
        }
        prior = __shfl_sync(0xffffffffu, prior, leader);
        r_reg[r] = valid ? prior + __popc(peers & lt_mask) : 0xffffffffu;
        __syncwarp();
    }
    __syncthreads();
    // Exclusive scan over the warps of each digit (earlier warps hold
    // earlier keys), then over the digits of the tile.
    uint32_t dcount = 0;
    if (tid < bins) {
#pragma unroll
        for (int w = 0; w < S::kWarps; ++w) {
            const uint32_t c = wcnt[w][tid];
            wcnt[w][tid] = dcount;
            dcount += c;
        }
    }
    {
        uint32_t all;
        const uint32_t start = block_exclusive_scan<S::kWarps>(dcount, warp_sums, all);
        if (tid < bins) tile_start[tid] = start;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < S::kItems; ++r) {
        if (r_reg[r] == 0xffffffffu) continue;
        const uint32_t digit = (k_reg[r] >> shift) & mask;
        r_reg[r] += tile_start[digit] + wcnt[warp][digit];
    }
    __syncthreads();  // every counter read before the staging area overwrites them
#pragma unroll
    for (int r = 0; r < S::kItems; ++r) {
        if (r_reg[r] == 0xffffffffu) continue;
        skey[r_reg[r]] = k_reg[r];
        sval[r_reg[r]] = v_reg[r];
    }
    __syncthreads();
    // Staged tile in digit order: consecutive threads write consecutive
    // positions of each digit's run.
    const int count = min(S::kTile, n - tile_base);
    for (int k = tid; k < count; k += S::kThreads) {
        const uint32_t key = skey[k];
        const uint32_t digit = (key >> shift) & mask;
        const uint32_t dst = tile_off[digit] + (static_cast<uint32_t>(k) - tile_start[digit]);
        keys_out[dst] = key;
        vals_out[dst] = sval[k];
    }
}

// ---------------------------------------------------------------------------
// Sorts of up to kClusterSortMax keys: one cluster of kClusterCtas CTAs (the
// portable cluster size) does every pass in one launch.  CTA r holds sorted
// positions [r kCTile, (r + 1) kCTile) of the current pass in shared
// memory.  A pass ranks the CTA's keys by digit (warp match + per-warp
// counters, items in position order: stable), reads every CTA's digit
// histogram through distributed shared memory to place its runs, and
// writes each key straight into the shared memory of the CTA that holds its
// destination.  Two cluster barriers a pass: the histograms complete before
// any is read, and every key delivered (and every histogram read) before
// the next pass.  The last pass's CTAs write their slices out.  The result
// is the multi-launch sort's: stable by digit, earlier positions first.
// ---------------------------------------------------------------------------
namespace cg = cooperative_groups;
constexpr int kCThreads = 512, kCItems = 4, kCWarps = kCThreads / 32;
constexpr int kCTile = kCThreads * kCItems;  // 2,048 keys per CTA
constexpr int kClusterCtas = 8;
constexpr int kClusterSortMax = kCTile * kClusterCtas;
constexpr int kCWarpChunk = kCTile / kCWarps;  // 128 consecutive positions per warp

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kCThreads)
k_sort_cluster(const uint32_t* __restrict__ keys, uint32_t* __restrict__ sorted_keys,
               uint32_t* __restrict__ sorted_idx, int n, int passes, int bits_per_pass) {
    __shared__ uint32_t buf_k[2][kCTile], buf_v[2][kCTile];
    __shared__ uint16_t wcnt[kCWarps][kMaxBins];  // per-warp digit counts (<= 128 each)
    __shared__ uint32_t hist[kMaxBins];            // this CTA's digit counts
    __shared__ uint32_t run_off[kMaxBins];         // global start of this CTA's digit run
    __shared__ uint32_t warp_sums[kCWarps];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = static_cast<int>(cluster.block_rank());
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t mask = (1u << bits_per_pass) - 1u;
    const int bins = static_cast<int>(mask) + 1;
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        const int shift = p * bits_per_pass;
        uint32_t k_reg[kCItems], v_reg[kCItems], r_reg[kCItems];
#pragma unroll
        for (int r = 0; r < kCItems; ++r) {
            const int idx = warp * kCWarpChunk + r * 32 + lane;  // slot in the CTA
            const int pos = rank * kCTile + idx;
            if (pos < n) {
                k_reg[r] = p == 0 ? keys[pos] : buf_k[cur][idx];
                v_reg[r] = p == 0 ? static_cast<uint32_t>(pos) : buf_v[cur][idx];
            } else {
                k_reg[r] = 0u;
                v_reg[r] = 0u;
            }
        }
        for (int d = tid; d < bins; d += kCThreads) {
#pragma unroll
            for (int w = 0; w < kCWarps; ++w) wcnt[w][d] = 0;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kCItems; ++r) {
            const int pos = rank * kCTile + warp * kCWarpChunk + r * 32 + lane;
            const bool valid = pos < n;
            const uint32_t digit = valid ? (k_reg[r] >> shift) & mask : 0xffffffffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, digit);
            const int leader = __ffs(peers) - 1;
            uint32_t prior = 0;
            if (valid && lane == leader) {
                prior = wcnt[warp][digit];
                wcnt[warp][digit] = static_cast<uint16_t>(prior + __popc(peers));
            }
            prior = __shfl_sync(0xffffffffu, prior, leader);
            r_reg[r] = valid ? prior + __popc(peers & lt_mask) : 0xffffffffu;
            __syncwarp();
        }
        __syncthreads();
        // Per digit: exclusive scan over the warps (earlier warps hold
        // earlier positions) and the CTA's count.
        if (tid < bins) {
            uint32_t run = 0;
#pragma unroll
            for (int w = 0; w < kCWarps; ++w) {
                const uint32_t c = wcnt[w][tid];
                wcnt[w][tid] = static_cast<uint16_t>(run);
                run += c;
            }
            hist[tid] = run;
        }
        cluster.sync();  // every CTA's histogram complete
        {
            uint32_t total = 0u, before = 0u;
            if (tid < bins) {
                for (int q = 0; q < kClusterCtas; ++q) {
                    const uint32_t h = *cluster.map_shared_rank(&hist[tid], q);
                    total += h;
                    before += q < rank ? h : 0u;
                }
            }
            uint32_t all;
            const uint32_t dbase = block_exclusive_scan<kCWarps>(total, warp_sums, all);
            if (tid < bins) run_off[tid] = dbase + before;
        }
        __syncthreads();
        const int nxt = cur ^ 1;
#pragma unroll
        for (int r = 0; r < kCItems; ++r) {
            if (r_reg[r] == 0xffffffffu) continue;
            const uint32_t digit = (k_reg[r] >> shift) & mask;
            const uint32_t dst = run_off[digit] + wcnt[warp][digit] + r_reg[r];
            const int q = static_cast<int>(dst / kCTile), slot = static_cast<int>(dst % kCTile);
            *cluster.map_shared_rank(&buf_k[nxt][slot], q) = k_reg[r];
            *cluster.map_shared_rank(&buf_v[nxt][slot], q) = v_reg[r];
        }
        cluster.sync();  // every key delivered and every histogram read
        cur = nxt;
    }
    const int count = min(kCTile, n - rank * kCTile);
    for (int k = tid; k < count; k += kCThreads) {
        sorted_keys[rank * kCTile + k] = buf_k[cur][k];
        sorted_idx[rank * kCTile + k] = buf_v[cur][k];
    }
}

}  // namespace

SortPlan make_sort_plan(int n, uint64_t num_cells, int tile) {
    SortPlan p;
    p.n = n;
    if (tile == Small::kTile || tile == Large::kTile)
        p.tile = tile;
    else
        p.tile = n < kSmallTileBelow ? Small::kTile : Large::kTile;
    p.tiles = std::max(1, (n + p.tile - 1) / p.tile);
    int bits = 1;
    while (bits < 32 && (uint64_t(1) << bits) < num_cells) ++bits;
    p.passes = (bits + 7) / 8;
    p.bits_per_pass = (bits + p.passes - 1) / p.passes;
    p.bins = 1 << p.bits_per_pass;
    return p;
}

size_t sort_scratch_bytes(int max_n) {
    // Sized for the smaller tile, which any plan of up to max_n keys may use.
    const size_t tiles = std::max(1, (max_n + kSortMinTile - 1) / kSortMinTile);
    return (tiles * kMaxBins + kMaxBins) * sizeof(uint32_t);
}

int sort_kernel_count(const SortPlan& plan) {
    if (plan.n <= kClusterSortMax) return 1;
    return plan.passes * (plan.tiles <= kSumTilesMax ? 2 : 3);
}

namespace {
template <class S>
void sort_passes(const SortPlan& plan, const uint32_t* keys, uint32_t* sorted_keys,
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
        launch_k(k_upsweep<S>, plan.tiles, S::kThreads, st, kin, plan.n, shift, mask,
                 plan.tiles, hist, status);
        const bool sum_tiles = plan.tiles <= kSumTilesMax;
        if (!sum_tiles)
            launch_k(k_scan<S>, plan.bins, S::kThreads, st, hist, totals, plan.tiles, status);
        launch_k(k_downsweep<S>, plan.tiles, S::kThreads, st, kin, vin, kout, vout, plan.n,
                 shift, mask, plan.tiles, hist, totals, status, sum_tiles);
        kin = kout;
        vin = vout;
    }
}
}  // namespace

void launch_sort(const SortPlan& plan, const uint32_t* keys, uint32_t* sorted_keys,
                 uint32_t* sorted_idx, uint32_t* alt_keys, uint32_t* alt_idx, void* scratch,
                 const unsigned* status, cudaStream_t st) {
    if (plan.n <= kClusterSortMax) {
        // Nothing to sort is sorted: zero keys launch nothing.
        if (plan.n > 0)
            launch_k(k_sort_cluster, static_cast<unsigned>(kClusterCtas), kCThreads, st, keys,
                     sorted_keys, sorted_idx, plan.n, plan.passes, plan.bits_per_pass);
        return;
    }
    if (plan.tile == Small::kTile)
        sort_passes<Small>(plan, keys, sorted_keys, sorted_idx, alt_keys, alt_idx, scratch, status,
                           st);
    else
        sort_passes<Large>(plan, keys, sorted_keys, sorted_idx, alt_keys, alt_idx, scratch, status,
                           st);
}

}  // namespace pbf
