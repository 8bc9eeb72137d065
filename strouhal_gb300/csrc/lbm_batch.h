// Batched stepping: per-instance descriptors and launchers (lbm_batch.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "lbm_device.cuh"

namespace stro {

// One lattice of a batch. Device-resident, read-only during a launch.
struct BatchInstance {
    StepArgs a;               // step arguments (uin/ulid at ramp factor 1 when `ramp` is set)
    float uin_target;         // unramped targets, used with `ramp`
    float lid_target[3];
    const float* ramp;        // ramp factor per round (rounds [0, steps)), or nullptr
    int64_t t0;               // stepsDone when the batch starts
    int64_t steps;            // rounds this instance takes part in
    int32_t log_every;        // log sum |u|^2 every so many rounds (even, 0 = off)
    int32_t trace_cap;        // capacity of `trace`
    double* trace;            // kinetic-energy samples: trace[s] at round s * log_every
    int64_t probe_first;      // round of the first force probe (an odd step), -1 = none
    int32_t probe_period;     // rounds from one probe to the next (chunk + 2, even)
    int32_t probe_count;      // probes in this run
    double* samples;          // box forces, samples[3 k + d] for probe k
    uint32_t tile_begin;      // first tile of this instance in the batch tile list
    uint32_t ntiles;          // tiles of this instance
    uint32_t cells;           // nx * ny * nz
    // Tile layout. tiles_x == 0: tile t holds the cells t * threads ..
    // (t + 1) * threads - 1 in x-fastest order. Otherwise (lattices with walls
    // or solid fractions) tile t is the block (t % tiles_x, t / tiles_x %
    // tiles_y, z = t / (tiles_x tiles_y)) of blockDim.x x blockDim.y cells, as
    // in a single-lattice step, so that the tiles away from the walls hold
    // plain fluid only.
    uint32_t tiles_x;
    uint32_t tiles_y;
    // Exact division of a linear cell index (< 2^31) by nx and by ny:
    // n / d = (n * m) >> (32 + s) with s = ceil(log2 d), m = ceil(2^(32+s) / d).
    uint64_t div_nx_m, div_ny_m;
    uint32_t div_nx_s, div_ny_s;
};


// Grid-barrier and error state of the persistent launch (zeroed before each launch).
struct BatchCtl {
    unsigned arrived;
    unsigned generation;
    int error;                // 1: a barrier wait timed out
    int pad;
    long long error_round;
};

struct BatchArgs {
    const BatchInstance* inst;  // sorted by `steps`, longest first
    const uint16_t* tile_inst;  // instance (index into inst) of every tile
    int32_t count;
    int64_t max_steps;
    double* kepart;             // one kinetic-energy partial per tile
    double* fpart;              // three force partials per tile (probe rounds)
    BatchCtl* ctl;
    long long spin_limit;       // polls before a barrier wait gives up
};

// `probes`: some instance takes force probes in this run (geometry batches
// only; the probe-capable kernels are used then).
cudaError_t launch_batch_persistent(const BatchArgs& b, int half_storage, int geo, int feat,
                                    int probes, unsigned grid, dim3 block, cudaStream_t st);
cudaError_t launch_batch_round(const BatchArgs& b, int half_storage, int geo, int feat, int probes,
                               int64_t r, uint32_t tiles, dim3 block, cudaStream_t st);
// One round over two tile lists of a walled batch: `bulk` tiles on the
// wall-free kernels, `edge` tiles on the wall-aware ones (each list the
// active prefix of its instance-ordered tiles).
cudaError_t launch_batch_round_lists(const BatchArgs& b, int half_storage, int feat, int probes,
                                     int64_t r, const uint32_t* bulk, uint32_t nbulk,
                                     const uint32_t* edge, uint32_t nedge, dim3 block,
                                     cudaStream_t st);
cudaError_t launch_batch_fold(const BatchArgs& b, int64_t r, cudaStream_t st);
int batch_persistent_blocks_per_sm(int half_storage, int geo, int feat, int probes, dim3 block);

}  // namespace stro
