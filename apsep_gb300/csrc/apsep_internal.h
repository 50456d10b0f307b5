// apsep_internal.h -- layouts shared by the kernels and the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace apsep {

// Error bits in Counters::err (read back by apsep_plan_check).
enum : uint32_t {
    ERR_LOOKBACK_TIMEOUT = 1u,  // a predecessor range never published
    ERR_TMA_TIMEOUT = 2u,       // a bulk copy did not complete in time
    ERR_INTERNAL = 4u,          // a search invariant failed (bug)
};

// Look-back flag values (low 2 bits of a status word's tag).
enum : uint32_t { FLAG_AGG = 1u, FLAG_INCL = 2u };
constexpr uint32_t EPOCH_LIMIT = (1u << 30) - 1u;

// Run-to-run control block at the head of a plan's scratch.  Zeroed once at
// creation with epoch = 1; each run leaves it ready for the next (the last
// CTA resets the counters and advances the epoch), so runs need no memset
// and can be captured in a CUDA graph.
struct alignas(64) Counters {
    uint32_t range_counter;  // next dynamic range id
    uint32_t done;           // CTAs finished in the current run
    uint32_t epoch;          // tag of the current run's status words, 1..EPOCH_LIMIT
    uint32_t err;            // ERR_* bits, sticky until read
    uint32_t pad[12];
};

// Scratch of one run, carved from one device allocation (or the static
// array of apsep_run_noalloc) by carve_scratch().
struct RangeScratch {
    Counters* ctr;
    uint64_t* range_state;  // [max_ranges] look-back words: tag<<32 | key bits
    void* range_min;        // [max_ranges] key: min of each range
    void* tile_min;         // [cap_tiles]  key: min of each tile
    uint64_t* tile_rpre;    // [cap_tiles]  has<<32 | bits: min of the range's keys before the tile
    void* chunk_min;        // [cap_chunks] key: min of each 32-key chunk
    int32_t* tile_defcnt;   // [cap_tiles]  keys of the tile left for the range's second phase
    uint32_t* tile_defmask; // [cap_tiles * kMaxTileKeys/32] which keys (when 0 < count < tile)
    int cap_tiles;
    int max_ranges;
};

constexpr int kMinTileKeys = 4096;  // smallest tile of any configuration
constexpr int kMaxTileKeys = 4096;  // largest tile of any configuration
constexpr int kMaxRanges = 2048;    // persistent CTAs per run, upper bound

// Byte offsets of the scratch arrays for `capacity` keys (256-byte aligned).
struct ScratchOffsets {
    size_t state, rmin, tmin, rpre, cmin, dcnt, dmask, total;
    int64_t cap_tiles;
};
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr ScratchOffsets scratch_offsets(int64_t capacity) {
    ScratchOffsets o{};
    const int64_t cap = capacity > 0 ? capacity : 1;
    o.cap_tiles = (cap + kMinTileKeys - 1) / kMinTileKeys + 1;
    const size_t cap_chunks = (size_t)(cap + 31) / 32 + kMaxTileKeys / 32;
    o.state = align256(sizeof(Counters));
    o.rmin = align256(o.state + (size_t)kMaxRanges * 8);
    o.tmin = align256(o.rmin + (size_t)kMaxRanges * 4);
    o.rpre = align256(o.tmin + (size_t)o.cap_tiles * 4);
    o.cmin = align256(o.rpre + (size_t)o.cap_tiles * 8);
    o.dcnt = align256(o.cmin + cap_chunks * 4);
    o.dmask = align256(o.dcnt + (size_t)o.cap_tiles * 4);
    o.total = align256(o.dmask + (size_t)o.cap_tiles * (kMaxTileKeys / 32) * 4);
    return o;
}

// Bytes of scratch for `capacity` keys; when base != nullptr also fills *s.
size_t carve_scratch(void* base, int64_t capacity, RangeScratch* s);

struct RangeArgs {
    const void* d_in;
    int32_t* d_out;
    int n;
    int num_tiles;
    int tiles_per_range;
    int num_ranges;
    int tma_rows;            // floor(n/32): rows covered by the tensor maps (0 = no TMA)
    uint32_t spin_limit;     // bound on every device-side wait (polls)
    int skip_publish_range;  // fault injection: this range never publishes (-1 = off)
    RangeScratch s;
};

// A kernel configuration: threads per CTA x keys per thread.
struct TileConfig {
    int nt;
    int ipt;
};
constexpr int kNumTileConfigs = 2;
extern const TileConfig kTileConfigs[kNumTileConfigs];

// Launch one run.  Fills a.num_ranges / a.tiles_per_range from the
// configuration's occupancy on the current device.
cudaError_t launch_range(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& map_in,
                         const CUtensorMap& map_out, cudaStream_t stream);
cudaError_t range_prepare(int cfg);  // smem attributes + occupancy, current device

}  // namespace apsep
