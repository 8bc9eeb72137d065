// Row-staged step: bulk copies move lattice rows through shared memory in
// both directions, so neither the loads in flight nor the stores hold
// registers, and every shared-memory address is a fixed offset.
//
// The one-cell kernels keep 19 loads per thread in flight; with FP16 storage
// those are 2-byte requests and the step stays well short of the HBM roofline
// however many threads are resident. Here a block owns tiles of R consecutive
// rows (y0..y0+R-1 at one z), walks them in a persistent loop, and splits its
// warps by role:
//   producer (lane 0 of warp 0) issues the 19*R bulk loads of a tile
//       (cp.async.bulk, completion counted on the stage's `full` mbarrier),
//       waits on the stage's `done` mbarrier, writes the stage back with 19*R
//       bulk stores (global <- shared, one bulk group per tile), and refills
//       a stage once its stores have finished reading it;
//   consumers (warps 1..) wait on `full`, collide their cells from the stage,
//       write the results back into the same stage, and arrive on `done`.
// No block-wide barrier is taken inside the loop: a consumer warp waits only
// for data, the producer only for consumers or its own stores.
// Stage layout: [row r][segment i][x], nx elements per segment row.
//   even pass: segment i of row r is row (y0+r, z) of plane i. The cell reads
//              slot i at (x) and writes slot opp(i) at (x): segment opp(i).
//   odd pass : segment i of row r is row (y0+r-c_iy, z-c_iz) of plane opp(i),
//              the slots that direction i is gathered from, x shifted by
//              -c_ix (periodic within the row). Direction i is scattered to
//              slot i at x+c_ix of row (y0+r+c_iy, z+c_iz): element
//              (x+c_ix) of segment opp(i) of row r, the very element the cell
//              gathered direction opp(i) from.
// In both passes each cell writes exactly the stage elements it read, so the
// in-place update needs no barrier between reads and writes, and the stores
// return each segment to the global row it came from. In the AA pattern the
// slots a cell reads are the slots it writes, so tiles never share a row
// segment and nothing is read after it is written within a launch.
//
// Every mbarrier wait is bounded and also watches a shared abort flag: a side
// whose wait gives up raises the flag and records an error code, the other
// side leaves at its next poll, and the producer waits (bounded again) for
// the block's loads and stores in flight before it returns.
//
// Requirements (checked by the host): periodic lattice (no walls or solid
// fractions), row bytes nx*sizeof(S) a multiple of 16, ny a multiple of R,
// 32 to 256 consumer threads (a multiple of 32).
//
// Compiled twice like lbm_step.cu: STRO_ARITH=0 (stro::exact) and
// STRO_ARITH=1 (stro::fused); each copy exports one RowsLaunchers table.
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

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                 "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() {
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Wait until at most one committed store group is still reading shared memory.
__device__ __forceinline__ void bulk_wait_read_1() {
    asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}

// Wait until every committed store group has completed.
__device__ __forceinline__ void bulk_wait_all() {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `parity` of `bar`.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
    for (long long k = 0; k < limit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Global row index (z*ny + y) of segment i of tile row r.
template <int PARITY, int I>
__device__ __forceinline__ uint32_t seg_row(uint32_t y, uint32_t z, uint32_t ny, uint32_t nz) {
    if constexpr (PARITY == 0) {
        return z * ny + y;
    } else {
        const uint32_t sy = (dcy(I) > 0) ? (y == 0 ? ny - 1 : y - 1)
                                         : (dcy(I) < 0 ? (y == ny - 1 ? 0 : y + 1) : y);
        const uint32_t sz = (dcz(I) > 0) ? (z == 0 ? nz - 1 : z - 1)
                                         : (dcz(I) < 0 ? (z == nz - 1 ? 0 : z + 1) : z);
        return sz * ny + sy;
    }
}

// Plane of segment i: plane i (even pass) or opp(i) (odd pass).
template <int PARITY, int I>
constexpr int seg_plane() {
    return PARITY == 0 ? I : opp(I);
}

// Move one tile between global memory and a stage: loads (LOAD) or stores.
template <typename S, int PARITY, bool LOAD>
__device__ __forceinline__ void move_tile(const StepArgs& a, uint32_t nx, uint32_t tile,
                                          uint32_t R, S* stage, uint64_t* bar) {
    const uint32_t ny = uint32_t(a.ny), nz = uint32_t(a.nz);
    const uint32_t tiles_y = ny / R;
    const uint32_t z = tile / tiles_y, y0 = (tile % tiles_y) * R;
    const uint32_t row_bytes = nx * uint32_t(sizeof(S));
    S* f = static_cast<S*>(a.f);
    if constexpr (LOAD) mbar_expect_tx(bar, 19u * R * row_bytes);
    for (uint32_t r = 0; r < R; ++r) {
        S* srow = stage + size_t(r) * 19 * nx;
        sfor<0, 19>([&](auto I) {
            constexpr int i = I;
            S* g = f + uint64_t(seg_plane<PARITY, i>()) * a.plane +
                   uint64_t(seg_row<PARITY, i>(y0 + r, z, ny, nz)) * nx;
            if constexpr (LOAD) bulk_load(srow + size_t(i) * nx, g, row_bytes, bar);
            else bulk_store(g, srow + size_t(i) * nx, row_bytes);
        });
    }
}

template <typename S>
__device__ __forceinline__ float sld(const S* p);
template <>
__device__ __forceinline__ float sld<float>(const float* p) { return *p; }
template <>
__device__ __forceinline__ float sld<__half>(const __half* p) { return __half2float(*p); }

// Collide one cell of a stage in place. `row` points at the cell's stage row.
template <typename S, int PARITY, int FEAT>
__device__ __forceinline__ void cell_in_stage(const StepArgs& a, S* row, uint32_t nx, uint32_t x,
                                              uint32_t n) {
    float fh[19];
    uint32_t xm = x, xp = x;
    if constexpr (PARITY == 1) {
        xm = (x == 0) ? nx - 1 : x - 1;
        xp = (x == nx - 1) ? 0 : x + 1;
    }
    // gather: element x - c_ix of segment i
    sfor<0, 19>([&](auto I) {
        constexpr int i = I;
        const uint32_t sx = (PARITY == 1 && dcx(i) > 0) ? xm : ((PARITY == 1 && dcx(i) < 0) ? xp : x);
        fh[i] = sld<S>(row + size_t(i) * nx + sx);
    });
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    cell_force<FEAT>(a, n, Fx, Fy, Fz);
    float ntx = 0.f, nty = 0.f, ntz = 0.f;
    collide<FEAT, STRO_ARITH>(fh, a, int(x), 0.0f, Fx, Fy, Fz, ntx, nty, ntz);
    // scatter: direction i to element x + c_ix of segment opp(i)
    sfor<0, 19>([&](auto I) {
        constexpr int i = I;
        const uint32_t dx = (PARITY == 1 && dcx(i) > 0) ? xp : ((PARITY == 1 && dcx(i) < 0) ? xm : x);
        store_ddf<S>(row + size_t(opp(i)) * nx + dx, fh[i]);
    });
}

// Bounded wait for phase `parity` of `bar` that also gives up when the block's
// abort flag is raised. A wait that runs out raises the flag itself.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                              long long limit) {
    for (long long k = 0; k < limit; ++k) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

constexpr int kMaxConsumers = 256;

// NXC: compile-time row length (0 = a.nx at run time). blockDim.x = 32 + consumers.
template <typename S, int PARITY, int FEAT, int NXC>
__global__ void __launch_bounds__(kMaxConsumers + 32, FEAT == 2 ? 2 : 3)
    k_rows(const StepArgs a, uint32_t R, uint32_t nstage, int* error, long long limit) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t nx = NXC ? uint32_t(NXC) : uint32_t(a.nx);
    const uint32_t tiles_y = uint32_t(a.ny) / R;
    const uint32_t ntiles = tiles_y * uint32_t(a.nz);
    const size_t stage_bytes = (size_t(19) * R * nx * sizeof(S) + 127) / 128 * 128;
    // 256 B of control words: full[8], done[8], abort flag
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* done = full + 8;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem_raw + 128);
    auto stage = [&](uint32_t s) {
        return reinterpret_cast<S*>(smem_raw + 256 + size_t(s) * stage_bytes);
    };
    const uint32_t consumers = blockDim.x - 32;
    // limit: polls per wait on a copy or on the consumers (a copy completes in
    // microseconds); 0 gives up at the first wait. Loads still in flight after a
    // timeout are drained with a fixed limit of their own, so no copy lands in
    // the shared memory of a block that has returned.
    const long long drain_limit = 1ll << 22;
    // this block's tiles: blockIdx.x + q * gridDim.x, q < my
    const uint32_t my = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < nstage; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&done[s], consumers);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (threadIdx.x < 32) {
        if (threadIdx.x != 0) return;
        // ---- producer
        uint32_t issued = 0;
        for (; issued < nstage && issued < my; ++issued)
            move_tile<S, PARITY, true>(a, nx, blockIdx.x + issued * gridDim.x, R, stage(issued),
                                       &full[issued]);
        uint32_t q = 0;
        for (; q < my; ++q) {
            const uint32_t s = q % nstage;
            if (!wait_or_abort(&done[s], (q / nstage) & 1u, abort_flag, limit)) break;
            move_tile<S, PARITY, false>(a, nx, blockIdx.x + q * gridDim.x, R, stage(s), nullptr);
            bulk_commit();
            // refill the stage of tile q-1 once its stores have read it
            if (q >= 1 && issued < my) {
                bulk_wait_read_1();
                const uint32_t rs = issued % nstage;
                move_tile<S, PARITY, true>(a, nx, blockIdx.x + issued * gridDim.x, R, stage(rs),
                                           &full[rs]);
                ++issued;
            }
        }
        if (q < my) {
            atomicExch(error, 1);
            // loads still in flight: tiles q .. issued-1
            for (uint32_t t = q; t < issued; ++t)
                mbar_wait_bounded(&full[t % nstage], (t / nstage) & 1u, drain_limit);
        }
        bulk_wait_all();
        return;
    }
    // ---- consumers
    const uint32_t c = threadIdx.x - 32;
    const uint32_t r_first = c / nx, x_first = c % nx;
    const uint32_t dr = consumers / nx, dxs = consumers % nx;
    for (uint32_t q = 0; q < my; ++q) {
        const uint32_t s = q % nstage;
        if (!wait_or_abort(&full[s], (q / nstage) & 1u, abort_flag, limit)) {
            atomicExch(error, 1);
            return;
        }
        const uint32_t tile = blockIdx.x + q * gridDim.x;
        const uint32_t z = tile / tiles_y, y0 = (tile % tiles_y) * R;
        S* st = stage(s);
        uint32_t r = r_first, x = x_first;
        while (r < R) {
            const uint32_t n = (z * uint32_t(a.ny) + y0 + r) * nx + x;
            cell_in_stage<S, PARITY, FEAT>(a, st + size_t(r) * 19 * nx, nx, x, n);
            x += dxs;
            r += dr;
            if (x >= nx) {
                x -= nx;
                ++r;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&done[s]);
    }
}

constexpr size_t kMaxRowsSmem = 220 * 1024;  // largest stage set the variant accepts
constexpr size_t kRowsSmemTarget = 72 * 1024;  // aim: three resident blocks per SM

template <typename S>
size_t stage_bytes(int nx, int R) {
    return (size_t(19) * R * nx * sizeof(S) + 127) / 128 * 128;
}

// Stages per block: as many as fit the per-block target, at least 2, at most 8.
template <typename S>
uint32_t stages_for(int nx, int R) {
    const size_t sb = stage_bytes<S>(nx, R);
    size_t n = (kRowsSmemTarget - 256) / sb;
    if (n < 2) n = 2;
    if (n > 8) n = 8;
    return uint32_t(n);
}

template <typename S>
size_t rows_smem(int nx, int R) {
    return 256 + stages_for<S>(nx, R) * stage_bytes<S>(nx, R);
}

template <typename S, int PARITY, int FEAT>
const void* rows_fn(int nx) {
    if (nx == 256) return reinterpret_cast<const void*>(&k_rows<S, PARITY, FEAT, 256>);
    return reinterpret_cast<const void*>(&k_rows<S, PARITY, FEAT, 0>);
}

template <typename S>
const void* pick(int parity, int feat, int nx) {
    if (parity == 0)
        return feat == 2 ? rows_fn<S, 0, 2>(nx)
                         : (feat == 1 ? rows_fn<S, 0, 1>(nx) : rows_fn<S, 0, 0>(nx));
    return feat == 2 ? rows_fn<S, 1, 2>(nx) : (feat == 1 ? rows_fn<S, 1, 1>(nx) : rows_fn<S, 1, 0>(nx));
}

}  // namespace

bool rows_step_supported(int half_storage, int geo, bool probe, int nx, int ny, int threads,
                         int rows) {
    const size_t es = half_storage ? 2 : 4;
    if (geo || probe || rows < 1 || rows > 8 || ny % rows != 0) return false;
    const size_t smem = half_storage ? rows_smem<__half>(nx, rows) : rows_smem<float>(nx, rows);
    return (size_t(nx) * es) % 16 == 0 && smem <= kMaxRowsSmem && threads >= 32 &&
           threads <= kMaxConsumers && threads % 32 == 0;
}

// Resident blocks per SM of one kernel at one (threads, smem), cached: the
// attribute call and the occupancy query cost host time on every launch. The
// dynamic shared-memory limit of a kernel is raised once to kMaxRowsSmem, so a
// cached entry stays valid whatever size another lattice asked for since.
int rows_blocks_per_sm(const void* fn, int threads, size_t smem, cudaError_t* err) {
    struct Entry { const void* fn; int threads; size_t smem; int per_sm; };
    static thread_local Entry cache[64];
    static thread_local int used = 0;
    static thread_local const void* raised[32];
    static thread_local int nraised = 0;
    for (int k = 0; k < used; ++k)
        if (cache[k].fn == fn && cache[k].threads == threads && cache[k].smem == smem)
            return cache[k].per_sm;
    bool is_raised = false;
    for (int k = 0; k < nraised; ++k) is_raised = is_raised || raised[k] == fn;
    if (!is_raised) {
        *err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(kMaxRowsSmem));
        if (*err != cudaSuccess) return 0;
        if (nraised < 32) raised[nraised++] = fn;
    }
    int per_sm = 0;
    *err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    if (*err != cudaSuccess) return 0;
    if (used < 64) cache[used++] = Entry{fn, threads, smem, per_sm};
    return per_sm;
}

cudaError_t launch_rows_step(const StepArgs& a, int half_storage, int parity, int feat,
                             int threads, int rows, int sm_count, int* error, long long polls,
                             cudaStream_t st) {
    const void* fn = half_storage ? pick<__half>(parity, feat, a.nx) : pick<float>(parity, feat, a.nx);
    const size_t smem = half_storage ? rows_smem<__half>(a.nx, rows) : rows_smem<float>(a.nx, rows);
    uint32_t nstage = half_storage ? stages_for<__half>(a.nx, rows) : stages_for<float>(a.nx, rows);
    cudaError_t e = cudaSuccess;
    const int per_sm = rows_blocks_per_sm(fn, threads + 32, smem, &e);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint32_t ntiles = (uint32_t(a.ny) / uint32_t(rows)) * uint32_t(a.nz);
    uint32_t grid = uint32_t(per_sm) * uint32_t(sm_count);
    if (grid > ntiles) grid = ntiles;
    uint32_t R = uint32_t(rows);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = dim3(threads + 32, 1, 1);  // producer warp + consumers
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    void* args[] = {const_cast<StepArgs*>(&a), &R, &nstage, &error, &polls};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

const RowsLaunchers kRows = {&rows_step_supported, &launch_rows_step};

}  // namespace STRO_ARITH_NS
}  // namespace stro
