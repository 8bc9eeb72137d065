// Host-side launch interface of the device kernels (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "lbm_device.cuh"

namespace stro {

// Grid of the one-cell kernels: (ceil(nx/bx), ceil(ny/by), nz).
inline dim3 step_grid(const StepArgs& a, dim3 block) {
    return dim3((a.nx + block.x - 1) / block.x, (a.ny + block.y - 1) / block.y, a.nz);
}

// Block lists of the bulk / boundary split: list entry k names the lattice
// block (bx cells by by rows) with linear index bxi + gx * (byi + gy * z).
// The index is split by multiply-shift divisions (a block index is below
// 2^27: at most 2^32 cells, at least 32 per block), a few instructions per
// thread instead of two integer divisions.
struct ListGrid {
    uint64_t mx, my;  // division_magic of gx and gy
    uint32_t gx, gy, sx, sy;
};

// Grid of the lattice blocks of shape `block` (in cells).
inline ListGrid list_grid(const StepArgs& a, dim3 block) {
    ListGrid g;
    g.gx = (uint32_t(a.nx) + block.x - 1) / block.x;
    g.gy = (uint32_t(a.ny) + block.y - 1) / block.y;
    division_magic(g.gx, &g.mx, &g.sx);
    division_magic(g.gy, &g.my, &g.sy);
    return g;
}

// Block coordinates of the linear block index blk.
__device__ __forceinline__ void block_coords(uint32_t blk, const ListGrid& g, uint32_t& bxi,
                                             uint32_t& byi, uint32_t& z) {
    const uint32_t t = uint32_t((uint64_t(blk) * g.mx) >> (32 + g.sx));  // blk / gx
    z = uint32_t((uint64_t(t) * g.my) >> (32 + g.sy));                    // t / gy
    bxi = blk - t * g.gx;
    byi = t - z * g.gy;
}

// Block coordinates of the list entry of this CUDA block.
__device__ __forceinline__ void list_coords(const uint32_t* list, const ListGrid& g,
                                            uint32_t& bxi, uint32_t& byi, uint32_t& z) {
    block_coords(list[blockIdx.x], g, bxi, byi, z);
}

// Flag bit of a list entry of the pair kernels' merged bulk list: the block
// is an x-face block (block indices stay below 2^27).
constexpr uint32_t kListFaceBit = 0x80000000u;

// Launchers of the step kernels (lbm_step.cu), one table per arithmetic:
// exact::kStep (the reference's expressions as written) and fused::kStep
// (the fused-multiply-add collision).
struct StepLaunchers {
    // One AA pass over the lattice. block.x * block.y must be a multiple of 32
    // and at most 256; the grid is step_grid(a, block).
    cudaError_t (*step)(const StepArgs& a, int half_storage, int parity, int geo, int feat,
                        bool probe, dim3 block, cudaStream_t st);
    // Register-capped one-cell kernels for periodic lattices (block <= 128 threads).
    cudaError_t (*capped)(const StepArgs& a, int half_storage, int parity, int feat, dim3 block,
                          cudaStream_t st);
    // One pass split over three block lists of the (bx,by) grid: `bulk` blocks
    // (every cell fluid, no wall neighbour, no solid fraction) run the
    // wall-free kernels at feature level feat_bulk, `face` blocks (walls only
    // in velocity-inflow columns at x = 0 / x = nx - 1, no solid fraction;
    // GEO 2) the x-face kernels at feat_bulk, `edge` blocks the wall-aware
    // kernels at feat_edge. Each cell touches only its own slots, so the
    // launches are independent. edge_colmajor: the edge blocks of the odd
    // pass take their cells column by column (a warp covers whole columns of
    // the block) instead of row by row. merged: `bulk` holds the bulk and the
    // x-face blocks in block order (x-face entries flagged kListFaceBit), run
    // in one launch; face / nface are unused.
    cudaError_t (*split)(const StepArgs& a, int half_storage, int parity, int feat_bulk,
                         int feat_edge, dim3 block, const uint32_t* bulk, uint32_t nbulk,
                         const uint32_t* face, uint32_t nface, const uint32_t* edge,
                         uint32_t nedge, int edge_colmajor, int merged, cudaStream_t st);
};

// Row-staged step (lbm_rows.cu): tiles of `rows` whole lattice rows move
// through shared memory by bulk loads and bulk stores, `threads` computing
// threads per block plus one copy warp, persistent over tiles. `error`
// receives 1 if a bounded wait gave up; `polls` bounds every wait (0: give up
// at the first one).
struct RowsLaunchers {
    bool (*supported)(int half_storage, int geo, bool probe, int nx, int ny, int threads,
                      int rows);
    cudaError_t (*launch)(const StepArgs& a, int half_storage, int parity, int feat, int threads,
                          int rows, int sm_count, int* error, long long polls, cudaStream_t st);
};

// FP16 periodic step with x-adjacent cell pairs per thread (lbm_pair.cu).
// block.x threads cover 2*block.x cells of a row.
struct PairLaunchers {
    bool (*supported)(int half_storage, int geo, bool probe, int nx, uint64_t plane, dim3 block);
    cudaError_t (*launch)(const StepArgs& a, int parity, int feat, dim3 block, cudaStream_t st);
    // Wide form: `cells` = 4 or 8 cells per thread (8- or 16-byte words),
    // block = bx threads along x (a multiple of 32 dividing nx / cells) by
    // `by` rows (dividing ny).
    bool (*wide_supported)(int half_storage, int geo, bool probe, int nx, int ny, uint64_t plane,
                           dim3 block, int cells);
    cudaError_t (*wide_launch)(const StepArgs& a, int parity, int feat, dim3 block, int cells,
                               cudaStream_t st);
    // Bulk and x-face blocks of the split in one launch, FP16 storage,
    // block.x / 2 by block.y threads per lattice block of shape `block` (in
    // cells): bulk blocks two x-adjacent cells per thread in 4-byte words,
    // blocks whose entry carries kListFaceBit the x-face code, two cells per
    // thread one after the other. Honours StepArgs::f_out.
    bool (*list_supported)(int half_storage, int feat, int nx, uint64_t plane, dim3 block);
    cudaError_t (*list_launch)(const StepArgs& a, int parity, int feat, dim3 block,
                               const uint32_t* list, uint32_t count, cudaStream_t st);
};

namespace exact {
extern const StepLaunchers kStep;
extern const RowsLaunchers kRows;
extern const PairLaunchers kPair;
}  // namespace exact
namespace fused {
extern const StepLaunchers kStep;
extern const RowsLaunchers kRows;
extern const PairLaunchers kPair;
}  // namespace fused



// Fields and reductions (lbm_probe.cu). `plane` is the DDF plane stride in
// elements, N the cell count. Reductions write per-block FP64 partials to
// `partials` and then fold them in a fixed order into `out`.
struct FieldView {
    void* f;
    uint64_t plane;
    uint32_t nx, ny, nz, N;
    const uint8_t* cell;    // nullptr: all fluid
    const float* ffield;    // nullptr: no force field
    float fx, fy, fz;       // uniform force
};

// Blocks of a fixed-order FP64 reduction over `count` items (depends on the
// count only): one per 1,024, at most kReductionMaxBlocks (which sizes every
// partials buffer).
constexpr int kReductionMaxBlocks = 2048;
int reduction_blocks(uint64_t count);

cudaError_t launch_init_field(const FieldView& v, int half_storage, uint32_t mode,
                              float amplitude, float tau, cudaStream_t st);
cudaError_t launch_moments(const FieldView& v, int half_storage, float4* out, cudaStream_t st);
// |u| colormap of slice z into nx*ny RGBA binary16 texels (colorize, Kernels.metal:476-500).
cudaError_t launch_render(const FieldView& v, int half_storage, const float* eps, uint32_t z,
                          float uref, __half* out, cudaStream_t st);
// out[0] = sum |u|^2, out[1] = sum 2 nu S:S (lattice units)
cudaError_t launch_observables(const FieldView& v, int half_storage, float omega,
                               double* partials, double* out, cudaStream_t st);
cudaError_t launch_mass(const FieldView& v, int half_storage, double* partials, double* out,
                        cudaStream_t st);
// out[0] = number of non-finite DDFs (as a double)
cudaError_t launch_nonfinite(const FieldView& v, int half_storage, double* partials, double* out,
                             cudaStream_t st);
// Sum nblocks x K partials in a fixed order into out[K].
cudaError_t launch_fold(const double* partials, int nblocks, int K, double* out, cudaStream_t st);

}  // namespace stro
