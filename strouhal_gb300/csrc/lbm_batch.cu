// Batched stepping of many independent lattices of uneven size.
//
// The reference runs the rungs of a credibility ladder and its Mach anchors
// one after another on one queue (Ladder.swift:74-121). Here all instances
// advance together: every lattice is cut into tiles of one block each, the
// instances are sorted by step count (longest first) so that the instances
// still running in round r are a prefix of the list and so are their tiles,
// and each round processes the active prefix. A tile is a run of consecutive
// cells in the instance's linear index (x fastest), so one block size fits
// every instance without idle threads, whatever its edge length; the only
// partial tile is an instance's last one. A table gives each tile's instance.
//
// Two launch forms, both captured in a CUDA graph by the host:
//   k_batch_persistent  one cooperative launch; blocks loop over rounds and
//                       meet at a grid barrier between rounds. Every wait is
//                       bounded: after `spin_limit` polls the block records a
//                       timeout in the control word and returns, and the other
//                       blocks leave at their next barrier.
//   k_batch_round       one launch per round over the active tiles (the graph
//                       holds the rounds in order; kernel boundaries are the
//                       barriers).
// The persistent kernel reads DDFs with ordinary (L1-cached) loads: a slot
// another SM wrote in the previous round is read only after the grid barrier,
// whose release / acquire pattern (gpu-scope fences around the arrival and
// generation atomics, then a block barrier) makes that write visible to every
// thread of the block, the same ordering a cooperative grid sync gives. Within
// a round no slot is read by one thread and written by another.
//
// Optional per-instance kinetic-energy traces are fused into the even pass:
// on a logging round each tile reduces sum |u|^2 of its cells (FP64, fixed
// order) into one partial, and the partials of an instance are folded in tile
// order after the round, so a trace is bitwise reproducible.
//
// Force probes (the sampled runs of a credibility ladder, Ladder.swift:54-66)
// work the same way on the odd pass: on an instance's probe round each tile
// reduces the momentum-exchange force of its boundary cells inside the
// instance's box into three FP64 partials, folded in tile order into the
// instance's sample buffer after the round.
#include "lbm_batch.h"
#include "lbm_cell.cuh"

namespace stro {

namespace {

// Descriptor of the instance owning `tile`, copied into registers: one table
// load finds the instance, and the step kernels then read its fields from
// the local copy (a reference into global memory would have to be reloaded
// after every DDF store, which the compiler cannot prove does not alias it).
__device__ __forceinline__ BatchInstance tile_instance(const BatchArgs& b, uint32_t tile) {
    return b.inst[b.tile_inst[tile]];
}

__device__ __forceinline__ uint32_t active_tiles(const BatchArgs& b, int64_t r) {
    uint32_t tiles = 0;
    for (int k = 0; k < b.count; ++k) {
        if (b.inst[k].steps <= r) break;
        tiles = b.inst[k].tile_begin + b.inst[k].ntiles;
    }
    return tiles;
}

__device__ __forceinline__ bool logs_at(const BatchInstance& I, int64_t r) {
    return I.log_every > 0 && r < I.steps && (r % I.log_every) == 0 && ((I.t0 + r) & 1) == 0;
}

__device__ __forceinline__ bool probes_at(const BatchInstance& I, int64_t r) {
    if (I.probe_count <= 0 || r < I.probe_first) return false;
    const int64_t d = r - I.probe_first;
    return d % I.probe_period == 0 && d / I.probe_period < I.probe_count;
}

template <typename S, int GEO, int FEAT, bool PROBES, bool CG>
__device__ __forceinline__ void process_tile(const BatchArgs& b, const BatchInstance& I,
                                             uint32_t tile, int64_t r) {
    const uint32_t tl = tile - I.tile_begin;
    int x, y, z;
    bool in;
    if (I.tiles_x != 0) {
        const uint32_t row = tl / I.tiles_x;
        x = int((tl - row * I.tiles_x) * blockDim.x + threadIdx.x);
        y = int((row % I.tiles_y) * blockDim.y + threadIdx.y);
        z = int(row / I.tiles_y);
        in = x < I.a.nx && y < I.a.ny;
    } else {
        const uint32_t lin = tl * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
        in = lin < I.cells;
        // multiply-shift division by nx and ny (exact for indices below 2^31)
        const uint32_t t = uint32_t((uint64_t(lin) * I.div_nx_m) >> (32 + I.div_nx_s));
        const uint32_t zz = uint32_t((uint64_t(t) * I.div_ny_m) >> (32 + I.div_ny_s));
        x = int(lin - t * uint32_t(I.a.nx));
        y = int(t - zz * uint32_t(I.a.ny));
        z = int(zz);
    }
    if (((I.t0 + r) & 1) == 0) {
        if (logs_at(I, r)) {
            float u2 = 0.0f;
            if (in) even_cell<S, GEO, FEAT, true, CG>(I.a, x, y, z, &u2);
            double v[1] = {(double)u2};
            block_reduce_store<1>(v, b.kepart + tile);
        } else if (in) {
            even_cell<S, GEO, FEAT, false, CG>(I.a, x, y, z);
        }
    } else {
        if constexpr (PROBES) {
            if (probes_at(I, r)) {
                double c[3] = {0.0, 0.0, 0.0};
                if (in) {
                    if (I.ramp != nullptr) {
                        const float rr = I.ramp[r];
                        const WallVel wv(I.uin_target * rr, I.lid_target[0] * rr,
                                         I.lid_target[1] * rr, I.lid_target[2] * rr);
                        odd_cell<S, GEO, FEAT, true, CG>(I.a, wv, x, y, z, c);
                    } else {
                        odd_cell<S, GEO, FEAT, true, CG>(I.a, WallVel(I.a), x, y, z, c);
                    }
                }
                block_reduce_store<3>(c, b.fpart + 3u * tile);
                return;
            }
        }
        if (!in) return;
        double dummy[3];
        if (I.ramp != nullptr) {
            const float rr = I.ramp[r];
            const WallVel wv(I.uin_target * rr, I.lid_target[0] * rr, I.lid_target[1] * rr,
                             I.lid_target[2] * rr);
            odd_cell<S, GEO, FEAT, false, CG>(I.a, wv, x, y, z, dummy);
        } else {
            odd_cell<S, GEO, FEAT, false, CG>(I.a, WallVel(I.a), x, y, z, dummy);
        }
    }
}

// Fold the kinetic-energy partials of every instance that logged in round r,
// and the force partials of every instance that probed in it, in tile order,
// into its trace or sample buffer. Called by one whole block.
__device__ void fold_round(const BatchArgs& b, int64_t r) {
    for (int k = 0; k < b.count; ++k) {
        const BatchInstance& I = b.inst[k];
        if (!logs_at(I, r)) continue;
        const int64_t s = r / I.log_every;
        double acc[1] = {0.0};
        const int tid = threadIdx.x + blockDim.x * threadIdx.y;
        const int nth = blockDim.x * blockDim.y;
        for (uint32_t t = tid; t < I.ntiles; t += nth) acc[0] += __ldcg(b.kepart + I.tile_begin + t);
        __shared__ double folded[1];
        block_reduce_store<1>(acc, folded);
        if (tid == 0 && s < I.trace_cap) I.trace[s] = folded[0];
        __syncthreads();
    }
    for (int k = 0; k < b.count; ++k) {
        const BatchInstance& I = b.inst[k];
        if (!probes_at(I, r)) continue;
        const int64_t s = (r - I.probe_first) / I.probe_period;
        double acc[3] = {0.0, 0.0, 0.0};
        const int tid = threadIdx.x + blockDim.x * threadIdx.y;
        const int nth = blockDim.x * blockDim.y;
        for (uint32_t t = tid; t < I.ntiles; t += nth) {
            const double* p = b.fpart + 3u * (I.tile_begin + t);
            acc[0] += __ldcg(p);
            acc[1] += __ldcg(p + 1);
            acc[2] += __ldcg(p + 2);
        }
        __shared__ double folded3[3];
        block_reduce_store<3>(acc, folded3);
        if (tid == 0) {
            I.samples[3 * s] = folded3[0];
            I.samples[3 * s + 1] = folded3[1];
            I.samples[3 * s + 2] = folded3[2];
        }
        __syncthreads();
    }
}

// Bounded grid barrier (sense by generation counter). Returns false when any
// block has recorded a timeout; the caller then returns.
__device__ bool grid_barrier(BatchCtl* ctl, unsigned& gen, long long spin_limit, int64_t r) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        const unsigned nblocks = gridDim.x;
        if (atomicAdd(&ctl->arrived, 1u) == nblocks - 1) {
            atomicExch(&ctl->arrived, 0u);
            __threadfence();
            atomicExch(&ctl->generation, gen + 1);
        } else {
            long long spins = 0;
            while (atomicAdd(&ctl->generation, 0u) == gen) {
                if (atomicAdd(&ctl->error, 0) != 0) break;
                if (++spins > spin_limit) {
                    if (atomicCAS(&ctl->error, 0, 1) == 0) ctl->error_round = r;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    ++gen;
    return *((volatile int*)&ctl->error) == 0;
}

template <typename S, int GEO, int FEAT, bool PROBES>
__global__ void __launch_bounds__(256) k_batch_persistent(const BatchArgs b) {
    unsigned gen = 0;
    for (int64_t r = 0; r < b.max_steps; ++r) {
        if (blockIdx.x == 0 && r > 0) fold_round(b, r - 1);
        const uint32_t tiles = active_tiles(b, r);
        for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
            const BatchInstance I = tile_instance(b, tile);
            process_tile<S, GEO, FEAT, PROBES, false>(b, I, tile, r);
        }
        if (!grid_barrier(b.ctl, gen, b.spin_limit, r)) return;
    }
    if (blockIdx.x == 0 && b.max_steps > 0) fold_round(b, b.max_steps - 1);
}

template <typename S, int GEO, int FEAT, bool PROBES>
__global__ void __launch_bounds__(256) k_batch_round(const BatchArgs b, int64_t r) {
    const uint32_t tile = blockIdx.x;
    const BatchInstance I = tile_instance(b, tile);
    process_tile<S, GEO, FEAT, PROBES, false>(b, I, tile, r);
}

// Rounds over a tile list: block i processes tile list[i]. The bulk tiles of
// a walled batch (only fluid cells without wall neighbours or solid
// fractions) run the wall-free kernel, the boundary tiles the wall-aware one,
// as the single-lattice bulk / boundary split does. In a probe round a bulk
// tile still stores its (zero) force partials, so the fold sees every tile.
// The wall-aware form is capped at 128 registers (two 256-thread blocks per
// SM instead of one; it spills a few words).
template <typename S, int GEO, int FEAT, bool PROBES>
__global__ void __launch_bounds__(256, GEO == 1 ? 2 : 0) k_batch_round_list(const BatchArgs b, int64_t r,
                                                          const uint32_t* list) {
    const uint32_t tile = list[blockIdx.x];
    const BatchInstance I = tile_instance(b, tile);
    process_tile<S, GEO, FEAT, PROBES, false>(b, I, tile, r);
}

__global__ void __launch_bounds__(256) k_batch_fold(const BatchArgs b, int64_t r) {
    fold_round(b, r);
}

template <typename S, int GEO, int FEAT, bool PROBES>
const void* persistent_fn() {
    return reinterpret_cast<const void*>(&k_batch_persistent<S, GEO, FEAT, PROBES>);
}

// Probe-capable kernels exist for geometry batches only: without walls or
// solid fractions nothing exchanges momentum and the host writes zero forces.
template <typename S>
const void* pick_persistent(int geo, int feat, int probes) {
    if (geo && probes)
        return feat == 2 ? persistent_fn<S, 1, 2, true>()
                         : (feat == 1 ? persistent_fn<S, 1, 1, true>()
                                      : persistent_fn<S, 1, 0, true>());
    if (geo)
        return feat == 2 ? persistent_fn<S, 1, 2, false>()
                         : (feat == 1 ? persistent_fn<S, 1, 1, false>()
                                      : persistent_fn<S, 1, 0, false>());
    return feat == 2 ? persistent_fn<S, 0, 2, false>()
                     : (feat == 1 ? persistent_fn<S, 0, 1, false>() : persistent_fn<S, 0, 0, false>());
}

template <typename S, int GEO, bool PROBES>
void launch_round_feat(const BatchArgs& b, int feat, int64_t r, uint32_t tiles, dim3 block,
                       cudaStream_t st) {
    if (feat == 2) k_batch_round<S, GEO, 2, PROBES><<<tiles, block, 0, st>>>(b, r);
    else if (feat == 1) k_batch_round<S, GEO, 1, PROBES><<<tiles, block, 0, st>>>(b, r);
    else k_batch_round<S, GEO, 0, PROBES><<<tiles, block, 0, st>>>(b, r);
}

template <typename S, int GEO, bool PROBES>
void launch_list_feat(const BatchArgs& b, int feat, int64_t r, const uint32_t* list,
                      uint32_t count, dim3 block, cudaStream_t st) {
    if (feat == 2) k_batch_round_list<S, GEO, 2, PROBES><<<count, block, 0, st>>>(b, r, list);
    else if (feat == 1) k_batch_round_list<S, GEO, 1, PROBES><<<count, block, 0, st>>>(b, r, list);
    else k_batch_round_list<S, GEO, 0, PROBES><<<count, block, 0, st>>>(b, r, list);
}

template <typename S>
cudaError_t launch_lists_typed(const BatchArgs& b, int feat, int probes, int64_t r,
                               const uint32_t* bulk, uint32_t nbulk, const uint32_t* edge,
                               uint32_t nedge, dim3 block, cudaStream_t st) {
    if (nbulk) {
        if (probes) launch_list_feat<S, 0, true>(b, feat, r, bulk, nbulk, block, st);
        else launch_list_feat<S, 0, false>(b, feat, r, bulk, nbulk, block, st);
    }
    if (nedge) {
        if (probes) launch_list_feat<S, 1, true>(b, feat, r, edge, nedge, block, st);
        else launch_list_feat<S, 1, false>(b, feat, r, edge, nedge, block, st);
    }
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_round_typed(const BatchArgs& b, int geo, int feat, int probes, int64_t r,
                               uint32_t tiles, dim3 block, cudaStream_t st) {
    if (geo && probes) launch_round_feat<S, 1, true>(b, feat, r, tiles, block, st);
    else if (geo) launch_round_feat<S, 1, false>(b, feat, r, tiles, block, st);
    else launch_round_feat<S, 0, false>(b, feat, r, tiles, block, st);
    return cudaGetLastError();
}

}  // namespace

const void* batch_persistent_kernel(int half_storage, int geo, int feat, int probes) {
    return half_storage ? pick_persistent<__half>(geo, feat, probes)
                        : pick_persistent<float>(geo, feat, probes);
}

cudaError_t launch_batch_persistent(const BatchArgs& b, int half_storage, int geo, int feat,
                                    int probes, unsigned grid, dim3 block, cudaStream_t st) {
    const void* fn = batch_persistent_kernel(half_storage, geo, feat, probes);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {const_cast<BatchArgs*>(&b)};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

cudaError_t launch_batch_round(const BatchArgs& b, int half_storage, int geo, int feat, int probes,
                               int64_t r, uint32_t tiles, dim3 block, cudaStream_t st) {
    if (tiles == 0) return cudaSuccess;
    return half_storage ? launch_round_typed<__half>(b, geo, feat, probes, r, tiles, block, st)
                        : launch_round_typed<float>(b, geo, feat, probes, r, tiles, block, st);
}

cudaError_t launch_batch_round_lists(const BatchArgs& b, int half_storage, int feat, int probes,
                                     int64_t r, const uint32_t* bulk, uint32_t nbulk,
                                     const uint32_t* edge, uint32_t nedge, dim3 block,
                                     cudaStream_t st) {
    return half_storage
               ? launch_lists_typed<__half>(b, feat, probes, r, bulk, nbulk, edge, nedge, block, st)
               : launch_lists_typed<float>(b, feat, probes, r, bulk, nbulk, edge, nedge, block, st);
}

cudaError_t launch_batch_fold(const BatchArgs& b, int64_t r, cudaStream_t st) {
    k_batch_fold<<<1, 256, 0, st>>>(b, r);
    return cudaGetLastError();
}

int batch_persistent_blocks_per_sm(int half_storage, int geo, int feat, int probes, dim3 block) {
    int n = 0;
    const void* fn = batch_persistent_kernel(half_storage, geo, feat, probes);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, int(block.x * block.y * block.z), 0) !=
        cudaSuccess)
        return 0;
    return n;
}

}  // namespace stro
