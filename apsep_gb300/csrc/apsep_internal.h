// apsep_internal.h -- layouts shared by the kernels and the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace apsep {

// Error bits in Counters::err (read back by apsep_plan_check).
enum : uint32_t {
    ERR_LOOKBACK_TIMEOUT = 1u,  // a predecessor tile never published
    ERR_TMA_TIMEOUT = 2u,       // a bulk copy did not complete in time
    ERR_INTERNAL = 4u,          // a search invariant failed (bug)
};

// Look-back flag values (low 2 bits of a status word's tag).
enum : uint32_t { FLAG_AGG = 1u, FLAG_INCL = 2u };
constexpr uint32_t EPOCH_LIMIT = (1u << 30) - 1u;

// Run-to-run control block at the head of a plan's scratch.  Zeroed once at
// plan creation (epoch starts at 1 by convention of the launcher); each run
// leaves it ready for the next, so runs need no memset and can be captured
// in a CUDA graph.
struct alignas(64) Counters {
    uint32_t tile_counter;  // next dynamic tile id
    uint32_t done;          // CTAs finished in the current run
    uint32_t epoch;         // tag of the current run's status words, 1..EPOCH_LIMIT
    uint32_t err;           // ERR_* bits, sticky until read
    uint32_t pad[12];
};

// Per-plan scratch (one device allocation, carved by the host).
struct TileScratch {
    Counters* ctr;
    uint64_t* state;     // [cap_tiles] decoupled look-back words: tag<<32 | key bits
    void* tile_min;      // [cap_tiles] key: min of each tile
    void* chunk_min;     // [cap_tiles * tile/32] key: min of each 32-key chunk
    int cap_tiles;
};

struct SingleArgs {
    const void* d_in;
    int32_t* d_out;
    int n;
    int num_tiles;
    int tma_rows;        // floor(n/32): rows covered by the tensor maps (0 = no TMA)
    uint32_t spin_limit; // bound on every device-side wait (polls)
    int skip_publish_tile;  // fault injection: this tile never publishes (-1 = off)
    TileScratch s;
};

// A tile-kernel configuration: threads per CTA x keys per thread.
struct TileConfig {
    int nt;
    int ipt;
};

// Launchers (apsep_single.cu).  cfg indexes kTileConfigs.
constexpr int kNumTileConfigs = 3;
extern const TileConfig kTileConfigs[kNumTileConfigs];

cudaError_t launch_single(int dtype, int incl, int cfg, const SingleArgs& a, const CUtensorMap& map_in,
                          const CUtensorMap& map_out, cudaStream_t stream);
size_t single_smem_bytes(int cfg);
cudaError_t single_prepare(int cfg);  // sets smem attributes on the current device

}  // namespace apsep
