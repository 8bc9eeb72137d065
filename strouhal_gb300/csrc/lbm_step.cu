// The D3Q19 AA-pattern fused stream-collide step for sm_103a.
//
// Restates the reference's `step` kernel (Kernels.metal:230-355) and its
// `collide` (Kernels.metal:105-228) as two kernels, one per AA parity:
//   even: read slot i of cell n, collide, write slot opp(i) of cell n;
//   odd : read slot opp(i) of n - c_i (or slot i of n behind a wall), collide,
//         write slot i of n + c_i (or slot opp(i) of n toward a wall).
// Each slot has one reader and one writer per pass and they are the same
// thread, so the update is in place and race-free with no atomics.
//
// Arithmetic contract: this file is compiled with -fmad=false and the only
// fused multiply-add is the explicit one of the reference (Kernels.metal:181),
// divisions and square roots are IEEE-rounded, and every expression keeps the
// reference's operation order. The results are therefore equal in value to
// the reference arithmetic evaluated in FP32 (only zero terms are skipped).
//
// Specialisations (all value-preserving):
//   GEO  = 0 periodic all-fluid box: no cell bytes, masks or wall logic;
//          1 walls and/or partially saturated cells;
//          2 (block lists only) blocks whose only walls are velocity-inflow
//            columns at x = 0 and x = nx - 1: wall links from x alone;
//          3 (block lists only) a merged list of GEO 0 and GEO 2 blocks.
//   FEAT = 0 lean collide: no sponge, LES, body force or NT cells;
//          1 sponge, body force, NT cells, each behind a uniform or per-cell branch;
//          2 also the Smagorinsky LES block;
//          3 the KBC collision instead of SRT / TRT (sponge and body force).
//   PROBE  odd pass with momentum-exchange force accumulation, reduced per
//          block in FP64 in a fixed order (no per-cell force buffer).
//
// The file is compiled twice: with STRO_ARITH=0 (namespace stro::exact, the
// reference arithmetic above) and with STRO_ARITH=1 (namespace stro::fused,
// the fused-multiply-add collision of lbm_cell.cuh). Each copy exports its
// launchers through one StepLaunchers table.
#include "lbm_cell.cuh"
#include "lbm_launch.h"

#ifndef STRO_ARITH
#define STRO_ARITH 0
#endif
#if STRO_ARITH == 0
#define STRO_ARITH_NS exact
#else
#define STRO_ARITH_NS fused
#endif

namespace stro {
namespace STRO_ARITH_NS {

// ---------------------------------------------------------------- kernels
// The KBC collision (FEAT 3) is capped at 80 registers (three blocks of 256
// per SM, a few spilled words): 31.6 GLUPS on the FP16 256^3 TGV against
// 29.1 at the compiler's 93/114. The other levels keep the compiler's choice.
template <typename S, int GEO, int FEAT>
__global__ void __launch_bounds__(256, FEAT == 3 ? 3 : 0) k_step_even(const StepArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.nx || y >= a.ny) return;
    even_cell<S, GEO, FEAT, false, false, STRO_ARITH>(a, x, y, blockIdx.z);
}

template <typename S, int GEO, int FEAT, bool PROBE>
__global__ void __launch_bounds__(256, FEAT == 3 && GEO == 0 ? 3 : 0) k_step_odd(const StepArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    double contrib[3] = {0.0, 0.0, 0.0};
    if constexpr (!PROBE) {
        if (x >= a.nx || y >= a.ny) return;
        odd_cell<S, GEO, FEAT, false, false, STRO_ARITH>(a, WallVel(a), x, y, blockIdx.z, contrib);
    } else {
        if (x < a.nx && y < a.ny)
            odd_cell<S, GEO, FEAT, true, false, STRO_ARITH>(a, WallVel(a), x, y, blockIdx.z, contrib);
        const uint32_t blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        block_reduce_store<3>(contrib, a.partials + 3u * blk);
    }
}

// Register-capped periodic kernels (64 registers, up to 8 blocks of 128 per
// SM): more warps in flight for the latency-bound FP16 case, at the price of
// a few spilled bytes. Same per-cell code.
template <typename S, int FEAT>
__global__ void __launch_bounds__(128, 8) k_step_even_capped(const StepArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.nx || y >= a.ny) return;
    even_cell<S, 0, FEAT, false, false, STRO_ARITH>(a, x, y, blockIdx.z);
}

template <typename S, int FEAT>
__global__ void __launch_bounds__(128, 8) k_step_odd_capped(const StepArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.nx || y >= a.ny) return;
    double contrib[3];
    odd_cell<S, 0, FEAT, false, false, STRO_ARITH>(a, WallVel(a), x, y, blockIdx.z, contrib);
}

template <typename S, int FEAT>
static void launch_capped_level(const StepArgs& a, int parity, dim3 grid, dim3 block,
                                cudaStream_t st) {
    if (parity == 0) k_step_even_capped<S, FEAT><<<grid, block, 0, st>>>(a);
    else k_step_odd_capped<S, FEAT><<<grid, block, 0, st>>>(a);
}

cudaError_t launch_step_capped(const StepArgs& a, int half_storage, int parity, int feat,
                               dim3 block, cudaStream_t st) {
    if (block.x * block.y > 128) return cudaErrorInvalidValue;
    const dim3 grid((a.nx + block.x - 1) / block.x, (a.ny + block.y - 1) / block.y, a.nz);
    if (half_storage) {
        if (feat == 2) launch_capped_level<__half, 2>(a, parity, grid, block, st);
        else if (feat == 1) launch_capped_level<__half, 1>(a, parity, grid, block, st);
        else launch_capped_level<__half, 0>(a, parity, grid, block, st);
    } else {
        if (feat == 2) launch_capped_level<float, 2>(a, parity, grid, block, st);
        else if (feat == 1) launch_capped_level<float, 1>(a, parity, grid, block, st);
        else launch_capped_level<float, 0>(a, parity, grid, block, st);
    }
    return cudaGetLastError();
}

// Block-list launches: block i of the grid processes lattice block list[i]
// (ListGrid, lbm_launch.h). Used to run the bulk of a walled lattice with the
// wall-free kernels and only its boundary blocks with the wall-aware ones.
__device__ __forceinline__ void list_block(const uint32_t* list, const ListGrid& g, int& x,
                                           int& y, int& z) {
    uint32_t bxi, byi, bz;
    list_coords(list, g, bxi, byi, bz);
    x = int(bxi * blockDim.x + threadIdx.x);
    y = int(byi * blockDim.y + threadIdx.y);
    z = int(bz);
}

// GEO 3: a merged list of bulk and x-face blocks in block order (x-face
// entries flagged kListFaceBit); each block runs the GEO 0 or GEO 2 code, a
// block-uniform branch. A 128-byte line shared by an x-face block and the
// bulk block beside it is then fetched from DRAM once: from separate
// launches each fetched the whole line for its half.
__device__ __forceinline__ bool list_block_merged(const uint32_t* list, const ListGrid& g, int& x,
                                                  int& y, int& z) {
    const uint32_t e = list[blockIdx.x];
    uint32_t bxi, byi, bz;
    block_coords(e & ~kListFaceBit, g, bxi, byi, bz);
    x = int(bxi * blockDim.x + threadIdx.x);
    y = int(byi * blockDim.y + threadIdx.y);
    z = int(bz);
    return (e & kListFaceBit) != 0u;
}

template <typename S, int GEO, int FEAT, bool PO>
__global__ void __launch_bounds__(256) k_list_even(const StepArgs a, const uint32_t* list,
                                                   const ListGrid g) {
    int x, y, z;
    if constexpr (GEO == 3) {
        const bool face = list_block_merged(list, g, x, y, z);
        if (x >= a.nx || y >= a.ny || z >= a.nz) return;
        if (face) even_cell<S, 2, FEAT, false, false, STRO_ARITH, true, PO>(a, x, y, z);
        else even_cell<S, 0, FEAT, false, false, STRO_ARITH, true, PO>(a, x, y, z);
        return;
    }
    list_block(list, g, x, y, z);
    if (x >= a.nx || y >= a.ny || z >= a.nz) return;
    even_cell<S, GEO, FEAT, false, false, STRO_ARITH, true, PO>(a, x, y, z);
}

// Column-major cell order inside a block: thread t takes column t / by, row
// t % by, so a warp covers 32 / by whole columns of the tile instead of 32 / bx
// whole rows. On the boundary blocks of the odd pass this keeps a column of
// wall-adjacent cells (the cells next to an inflow wall at x = 0 or nx - 1)
// in warps of their own: the plain cells beside them no longer sit in warps
// that also run the moving-wall branches. The rows of a tile are re-read by
// its other warps, so the narrower warp accesses are served from L1.
__device__ __forceinline__ void list_block_colmajor(const uint32_t* list, const ListGrid& g,
                                                    int& x, int& y, int& z) {
    uint32_t bxi, byi, bz;
    list_coords(list, g, bxi, byi, bz);
    const uint32_t tid = threadIdx.x + blockDim.x * threadIdx.y;
    x = int(bxi * blockDim.x + tid / blockDim.y);
    y = int(byi * blockDim.y + tid % blockDim.y);
    z = int(bz);
}

template <typename S, int GEO, int FEAT, bool PO, bool COLMAJOR = false>
__global__ void __launch_bounds__(256) k_list_odd(const StepArgs a, const uint32_t* list,
                                                  const ListGrid g) {
    int x, y, z;
    if constexpr (GEO == 3) {
        const bool face = list_block_merged(list, g, x, y, z);
        if (x >= a.nx || y >= a.ny || z >= a.nz) return;
        if (face) {
            odd_cell_xface<S, FEAT, STRO_ARITH, PO>(a, WallVel(a), x, y, z);
        } else {
            double contrib[3];
            odd_cell<S, 0, FEAT, false, false, STRO_ARITH, true, PO>(a, WallVel(a), x, y, z,
                                                                     contrib);
        }
        return;
    }
    if constexpr (COLMAJOR) list_block_colmajor(list, g, x, y, z);
    else list_block(list, g, x, y, z);
    if (x >= a.nx || y >= a.ny || z >= a.nz) return;
    if constexpr (GEO == 2) {
        odd_cell_xface<S, FEAT, STRO_ARITH, PO>(a, WallVel(a), x, y, z);
    } else {
        double contrib[3];
        odd_cell<S, GEO, FEAT, false, false, STRO_ARITH, true, PO>(a, WallVel(a), x, y, z,
                                                                   contrib);
    }
}

// The wall-free and x-face lists address the planes through the 32-bit plane
// offsets when the lattice's 19 planes fit 2^32 elements (StepArgs::poff
// filled), the wall-aware list always through 64-bit plane products.
template <typename S, int GEO, int FEAT>
static void launch_list(const StepArgs& a, int parity, const uint32_t* list, uint32_t count,
                        dim3 block, bool colmajor, cudaStream_t st) {
    if (count == 0) return;
    const ListGrid g = list_grid(a, block);
    const bool po = GEO != 1 && a.poff[1] != 0;
    if (parity == 0) {
        if (po) k_list_even<S, GEO, FEAT, true><<<count, block, 0, st>>>(a, list, g);
        else k_list_even<S, GEO, FEAT, false><<<count, block, 0, st>>>(a, list, g);
    } else if (GEO == 1 && colmajor) {
        k_list_odd<S, GEO, FEAT, false, true><<<count, block, 0, st>>>(a, list, g);
    } else if (po) {
        k_list_odd<S, GEO, FEAT, true><<<count, block, 0, st>>>(a, list, g);
    } else {
        k_list_odd<S, GEO, FEAT, false><<<count, block, 0, st>>>(a, list, g);
    }
}

template <typename S, int GEO>
static void launch_list_level(const StepArgs& a, int parity, int feat, const uint32_t* list,
                              uint32_t count, dim3 block, bool colmajor, cudaStream_t st) {
    if (feat == 3) launch_list<S, GEO, 3>(a, parity, list, count, block, colmajor, st);
    else if (feat == 2) launch_list<S, GEO, 2>(a, parity, list, count, block, colmajor, st);
    else if (feat == 1) launch_list<S, GEO, 1>(a, parity, list, count, block, colmajor, st);
    else launch_list<S, GEO, 0>(a, parity, list, count, block, colmajor, st);
}

cudaError_t launch_step_split(const StepArgs& a, int half_storage, int parity, int feat_bulk,
                              int feat_edge, dim3 block, const uint32_t* bulk, uint32_t nbulk,
                              const uint32_t* face, uint32_t nface, const uint32_t* edge,
                              uint32_t nedge, int edge_colmajor, int merged, cudaStream_t st) {
    const bool col = edge_colmajor != 0;
    if (half_storage) {
        if (merged) {
            launch_list_level<__half, 3>(a, parity, feat_bulk, bulk, nbulk, block, false, st);
        } else {
            launch_list_level<__half, 0>(a, parity, feat_bulk, bulk, nbulk, block, false, st);
            launch_list_level<__half, 2>(a, parity, feat_bulk, face, nface, block, false, st);
        }
        launch_list_level<__half, 1>(a, parity, feat_edge, edge, nedge, block, col, st);
    } else {
        if (merged) {
            launch_list_level<float, 3>(a, parity, feat_bulk, bulk, nbulk, block, false, st);
        } else {
            launch_list_level<float, 0>(a, parity, feat_bulk, bulk, nbulk, block, false, st);
            launch_list_level<float, 2>(a, parity, feat_bulk, face, nface, block, false, st);
        }
        launch_list_level<float, 1>(a, parity, feat_edge, edge, nedge, block, col, st);
    }
    return cudaGetLastError();
}

// ----------------------------------------------------------------- launcher
template <typename S, int FEAT>
static void launch_level(const StepArgs& a, int parity, int geo, bool probe, dim3 grid, dim3 block,
                         cudaStream_t st) {
    if (parity == 0) {
        if (geo) k_step_even<S, 1, FEAT><<<grid, block, 0, st>>>(a);
        else k_step_even<S, 0, FEAT><<<grid, block, 0, st>>>(a);
    } else if (probe) {
        k_step_odd<S, 1, FEAT, true><<<grid, block, 0, st>>>(a);
    } else if (geo) {
        k_step_odd<S, 1, FEAT, false><<<grid, block, 0, st>>>(a);
    } else {
        k_step_odd<S, 0, FEAT, false><<<grid, block, 0, st>>>(a);
    }
}

template <typename S>
static cudaError_t launch_typed(const StepArgs& a, int parity, int geo, int feat, bool probe,
                                dim3 grid, dim3 block, cudaStream_t st) {
    if (probe && (parity == 0 || !geo)) return cudaErrorInvalidValue;
    if (feat == 3) launch_level<S, 3>(a, parity, geo, probe, grid, block, st);
    else if (feat == 2) launch_level<S, 2>(a, parity, geo, probe, grid, block, st);
    else if (feat == 1) launch_level<S, 1>(a, parity, geo, probe, grid, block, st);
    else launch_level<S, 0>(a, parity, geo, probe, grid, block, st);
    return cudaGetLastError();
}

cudaError_t launch_step(const StepArgs& a, int half_storage, int parity, int geo, int feat,
                        bool probe, dim3 block, cudaStream_t st) {
    const dim3 grid((a.nx + block.x - 1) / block.x, (a.ny + block.y - 1) / block.y, a.nz);
    if (half_storage) return launch_typed<__half>(a, parity, geo, feat, probe, grid, block, st);
    return launch_typed<float>(a, parity, geo, feat, probe, grid, block, st);
}

const StepLaunchers kStep = {&launch_step, &launch_step_capped, &launch_step_split};

}  // namespace STRO_ARITH_NS
}  // namespace stro
