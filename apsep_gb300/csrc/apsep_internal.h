// apsep_internal.h -- layouts shared by the kernels and the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "apsep.h"

namespace apsep {

// Error bits in Counters::err (read back by apsep_plan_check).
enum : uint32_t {
    ERR_LOOKBACK_TIMEOUT = 1u,  // a predecessor range never published
    ERR_TMA_TIMEOUT = 2u,       // a bulk copy did not complete in time
    ERR_INTERNAL = 4u,          // a search invariant failed (bug)
    ERR_BAD_OFFSETS = 8u,       // segment offsets not 0 = off[0] <= ... <= off[nseg] = n
};

// Look-back flag values (low 2 bits of a status word's tag).
enum : uint32_t { FLAG_AGG = 1u, FLAG_INCL = 2u };
constexpr uint32_t EPOCH_LIMIT = (1u << 30) - 1u;

// Run-to-run control block at the head of a plan's scratch.  Zeroed once at
// creation with epoch = 1; each run leaves it ready for the next (the last
// CTA resets the counters and advances the epoch), so runs need no memset
// and can be captured in a CUDA graph.
struct alignas(64) Counters {
    uint32_t range_counter;  // next dynamic range id (one range per warp)
    uint32_t done;           // warps finished in the current run
    uint32_t epoch;          // tag of the current run's status words, 1..EPOCH_LIMIT
    uint32_t err;            // ERR_* bits, sticky until read
    uint32_t finished;       // ranges that published their minimum in the current run
    uint32_t pad[11];
};

// Scratch of one run, carved from one device allocation (or the static
// array of apsep_run_noalloc) by carve_scratch().
struct RangeScratch {
    Counters* ctr;
    uint64_t* group_min;    // [max_ranges/32] atomic min of (EPOCH_LIMIT - epoch) << 32 | ordered key
                            //   over each group of 32 ranges; all-ones when created
    uint32_t* cta_ready;    // [kMaxCtas * kReadyStride] epoch in which every range has published, one line per CTA
    uint64_t* range_state;  // [max_ranges] tag<<32 | key bits: min of a finished range
    uint64_t* range_key;    // [max_ranges] 8-byte keys: the range minimum (range_state holds the tag)
    void* top_key;          // [max_ranges * kTopEntries] key: top of each range's final stack, bottom first
    int32_t* top_pos;       // [max_ranges * kTopEntries] their positions
    uint32_t* top_cnt;      // [max_ranges] entries published | bit 31: they are the whole stack
    void* tile_min;         // [cap_tiles]  key: min of each tile
    void* chunk_min;        // [cap_chunks] key: min of each 32-key chunk
    uint32_t* tile_flag;    // [cap_tiles]  flagged keys of the tile | bit 31: some are capped
    uint32_t* tile_mask;    // [cap_tiles * kMaxTileKeys/32] which keys are flagged
    int cap_tiles;
    int max_ranges;
};

constexpr int kMinTileKeys = 256;   // smallest tile of any configuration (one warp's)
constexpr int kMaxTileKeys = 512;   // largest tile of any configuration
constexpr int kMaxRanges = 4096;    // persistent warps per run, upper bound
constexpr int kMaxCtas = kMaxRanges / 4;  // every configuration runs >= 4 warps per CTA
constexpr int kReadyStride = 16;          // words between two CTAs' ready flags (64 bytes)
constexpr int kTopEntries = 32;           // stack entries each range publishes for later ranges

// Byte offsets of the scratch arrays for `capacity` keys (256-byte aligned).
struct ScratchOffsets {
    size_t gmin, ready, state, rkey, topk, topp, topc, tmin, cmin, flag, mask, total;
    int64_t cap_tiles;
};
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
// kb: bytes per key (4: int32 / float32; 8: int64 / float64).
constexpr ScratchOffsets scratch_offsets(int64_t capacity, int kb = 4) {
    ScratchOffsets o{};
    const int64_t cap = capacity > 0 ? capacity : 1;
    o.cap_tiles = (cap + kMinTileKeys - 1) / kMinTileKeys + 1;
    const size_t cap_chunks = (size_t)(cap + 31) / 32 + kMaxTileKeys / 32;
    o.gmin = align256(sizeof(Counters));
    o.ready = align256(o.gmin + (size_t)(kMaxRanges / 32) * 8);
    o.state = align256(o.ready + (size_t)kMaxCtas * kReadyStride * 4);
    o.rkey = align256(o.state + (size_t)kMaxRanges * 8);
    o.topk = align256(o.rkey + (size_t)kMaxRanges * 8);
    o.topp = align256(o.topk + (size_t)kMaxRanges * kTopEntries * kb);
    o.topc = align256(o.topp + (size_t)kMaxRanges * kTopEntries * 4);
    o.tmin = align256(o.topc + (size_t)kMaxRanges * 4);
    o.cmin = align256(o.tmin + (size_t)o.cap_tiles * kb);
    o.flag = align256(o.cmin + cap_chunks * kb);
    o.mask = align256(o.flag + (size_t)o.cap_tiles * 4);
    o.total = align256(o.mask + (size_t)o.cap_tiles * (kMaxTileKeys / 32) * 4);
    return o;
}

// The counters must start zeroed; a run leaves them zeroed, a run that timed
// out may not (apsep_plan_check clears them, keeping the epoch).
constexpr size_t control_bytes() { return sizeof(Counters); }
constexpr size_t group_min_bytes() { return (size_t)(kMaxRanges / 32) * 8; }

// Bytes of scratch for `capacity` keys of kb bytes; when base != nullptr also fills *s.
size_t carve_scratch(void* base, int64_t capacity, RangeScratch* s, int kb = 4);

struct RangeArgs {
    const void* d_in;
    int32_t* d_out;
    int n;
    int num_tiles;
    int tiles_per_range;
    int num_ranges;
    int tma_rows;            // floor(n/32): rows covered by the tensor maps (0 = no TMA)
    int head;                // 0..3 virtual keys in front of the array (d_in, d_out and n
                             //   include them) so that the TMA view starts 16-byte aligned;
                             //   never read or written, answers are relative to them
    uint32_t spin_limit;     // bound on every device-side wait (polls)
    int skip_publish_range;  // fault injection: this range never publishes (-1 = off)
    const int64_t* offsets;  // segmented runs: nseg + 1 segment offsets into d_in; else nullptr
    int nseg;
    RangeScratch s;
    int64_t* d_out64 = nullptr;  // int64 answers (the int64-position path's kernels): out_base + answer
    int64_t out_base = 0;
};

// Runs with int64 answers (RangeArgs::d_out64): a key that no key of the run
// answers reads UNRESOLVED64, and a tile whose keys are all unanswered within
// their range is not written at all; its tile_flag word carries
// TILE_NOT_STORED (phase 2 still writes the keys that it answers).
constexpr int64_t UNRESOLVED64 = -2;
// Output forms of a run (the engine's OUTM template parameter): int32
// answers; int64 answers (above); int32 spans, position - answer.
constexpr int OUT_I32 = 0, OUT_I64 = 1, OUT_SPAN = 2;
constexpr uint32_t TILE_NOT_STORED = 0x40000000u;

// The TMA view of a run: the number of virtual keys (0..3) in front of d_in
// that put the view on a 16-byte boundary, or -1 when the input and the output
// sit at different offsets within 16 bytes (no common view: plain loads and
// stores throughout).  Tile 0, which holds the virtual keys, always takes the
// plain path, so nothing in front of the arrays is touched.
inline int view_head(const void* d_in, const void* d_out) {
    const int hi = (int)((uintptr_t)d_in % 16 / 4), ho = (int)((uintptr_t)d_out % 16 / 4);
    return hi == ho ? hi : -1;
}

// A kernel configuration: warps per CTA x keys per lane (a warp's tile is 32*ipt keys).
struct TileConfig {
    int wpc;
    int ipt;
};
constexpr int kNumTileConfigs = 6;
extern const TileConfig kTileConfigs[kNumTileConfigs];

// Launch one run.  Fills a.num_ranges / a.tiles_per_range from the
// configuration's occupancy on the current device.
cudaError_t launch_range(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& map_in,
                         const CUtensorMap& map_out, cudaStream_t stream);
cudaError_t range_prepare(int cfg);  // smem attributes + occupancy, current device
// Segmented runs (a.offsets, a.nseg set): the same engine, answers relative to
// each key's segment start.
cudaError_t launch_range_segmented(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& map_in,
                                   const CUtensorMap& map_out, cudaStream_t stream);
// 8-byte keys (dtype 2: int64, 3: float64): one configuration (8 keys per
// lane, 8 warps per CTA), single arrays and segmented batches (RangeArgs::offsets).
constexpr int kWideTileKeys = 256;
cudaError_t prepare_wide();
cudaError_t launch_range_wide(int dtype, int incl, RangeArgs& a, const CUtensorMap& map_in,
                              const CUtensorMap& map_out, cudaStream_t st);

// A single array behind a view head (RangeArgs::head > 0): the segmented
// kernel with one implicit segment and the whole-tile early paths.
cudaError_t prepare_view(int cfg, int* ctas_per_sm);
cudaError_t launch_range_view(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& map_in,
                              const CUtensorMap& map_out, cudaStream_t st);
cudaError_t prepare_segmented(int cfg, int* ctas_per_sm);
cudaError_t range_max_warps(int cfg, int* warps);  // persistent warps of one launch, current device
// A single array (no view head) with int64 answers a.out_base + answer into
// a.d_out64 (4-byte keys in configuration 0, 8-byte keys in theirs); flagged keys
// get UNRESOLVED64 and all-deferred tiles are not written (TILE_NOT_STORED).
cudaError_t launch_range_out64(int dtype, int incl, RangeArgs& a, const CUtensorMap& map_in, cudaStream_t st);
// A single array (no view head, 4-byte keys) through the order-reversing key
// map in configuration 0: previous-greater answers (int32), or with span != 0
// (strict comparison only) the stock span, position - answer.
cudaError_t launch_range_flipped(int dtype, int incl, int span, RangeArgs& a, const CUtensorMap& map_in,
                                 const CUtensorMap& map_out, cudaStream_t st);
// A single array (no view head, 4-byte keys) seen reversed in configuration
// 0: next-smaller answers (n - 1 - the reversed run's answer, at the mirrored
// position), TMA tiles only when n is a multiple of 32 (a.tma_rows * 32 == n).
cudaError_t launch_range_reversed(int dtype, int incl, RangeArgs& a, const CUtensorMap& map_in,
                                  const CUtensorMap& map_out, cudaStream_t st);
// Arms one-shot fault injection for the next apsep_run_noalloc call.
void noalloc_debug_inject(int32_t range, uint32_t spin_limit);

}  // namespace apsep

struct apsep_plan;
// One single-array run of the plan with int64 answers (out_base + answer into
// d_out; see launch_range_out64): 4-byte keys in configuration 0, 8-byte keys
// in theirs, tiles by TMA when d_in is 16-byte aligned, else by plain loads.
// chunk_min, when not null, takes the run's minima of every 32 keys (in key
// order, up to the end of the last tile) instead of the plan's scratch.
// *layout returns the run's arguments: tile and range layout, scratch words.
// One single-array run of the plan through the order-reversing key map
// (launch_range_flipped): previous greater (span = 0) or the stock span
// (span = 1, APSEP_LT).  APSEP_ENOTSUP when the engine has no such form for
// the call (8-byte keys, keys or answers off a 16-byte boundary, answers over
// the keys): the caller then takes its general route.
apsep_status plan_run_flipped(struct apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                              int span, void* stream);
// One single-array run of the plan over the reversed array
// (launch_range_reversed): out[i] = the next j > i with a[j] < a[i] (<= under
// APSEP_LE), else -1.  APSEP_ENOTSUP when the engine has no such form for the
// call (8-byte keys, keys or answers off a 16-byte boundary, n not a multiple
// of 32, answers over the keys): the caller then takes its general route.
apsep_status plan_run_reversed(struct apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                               void* stream);
apsep_status plan_run_out64(struct apsep_plan* plan, const void* d_in, int64_t* d_out, int64_t n, int64_t out_base,
                            apsep_cmp cmp, void* chunk_min, void* stream, apsep::RangeArgs* layout);
