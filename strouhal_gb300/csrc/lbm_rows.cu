// Row-streaming step: TMA bulk copies stage lattice rows in shared memory.
//
// The one-cell kernels issue 19 dependent global loads per thread and then
// compute; with FP16 storage that keeps too few bytes in flight per SM and the
// step is latency-bound. Here each block owns whole rows (y, z) and walks them
// in a persistent loop. For every row one elected thread issues 19 bulk copies
// (cp.async.bulk, completion counted on an mbarrier) of the row segments the
// row needs into a shared-memory stage, NSTAGE rows ahead of the compute, so
// HBM reads proceed while the block collides the current row.
//   even pass: segment i = row (y, z) of plane i
//   odd pass : segment i = row (y - c_iy, z - c_iz) of plane opp(i); the x
//              shift (periodic within the row) is applied when reading smem.
// Results are stored straight from registers (even: slot opp(i) of the cell;
// odd: slot i of cell (x + c_ix mod nx, y + c_iy, z + c_iz)).
//
// Hazards: in the AA pattern every slot is read and written by the same cell
// in a pass, so a row prefetched ahead is never written before it is read, and
// no bulk copy reads memory written in the same launch.
// Every mbarrier wait is bounded; a wait that gives up records an error code
// in the control word, then waits (bounded again) for its block's own copies
// before returning, so no copy lands in shared memory after the block exits.
//
// Requirements (checked by the host): periodic lattice (no walls or solid
// fractions), row bytes nx*sizeof(S) a multiple of 16, 19 rows per stage in
// shared memory.
#include "lbm_cell.cuh"
#include "lbm_launch.h"

namespace stro {

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

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
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

template <typename S>
__device__ __forceinline__ float smem_ld(const S* p);
template <>
__device__ __forceinline__ float smem_ld<float>(const float* p) {
    return *p;
}
template <>
__device__ __forceinline__ float smem_ld<__half>(const __half* p) {
    return __half2float(*p);
}

// Issue the 19 segment copies of lattice row `row` into stage buffer `buf`.
template <typename S, int PARITY>
__device__ __forceinline__ void issue_row(const StepArgs& a, uint32_t row, S* buf, uint64_t* bar) {
    const uint32_t nx = uint32_t(a.nx), ny = uint32_t(a.ny), nz = uint32_t(a.nz);
    const uint32_t row_bytes = nx * sizeof(S);
    const S* f = static_cast<const S*>(a.f);
    const uint32_t y = row % ny, z = row / ny;
    mbar_expect_tx(bar, 19u * row_bytes);
    sfor<0, 19>([&](auto I) {
        constexpr int i = I;
        uint32_t src_row = row;
        int plane = i;
        if constexpr (PARITY == 1) {
            plane = opp(i);
            const uint32_t sy = uint32_t(int(y + ny) - dcy(i)) % ny;  // y - c_iy (mod ny)
            const uint32_t sz = uint32_t(int(z + nz) - dcz(i)) % nz;  // z - c_iz (mod nz)
            src_row = sz * ny + sy;
        }
        bulk_copy_g2s(buf + size_t(i) * nx, f + uint64_t(plane) * a.plane + uint64_t(src_row) * nx,
                      row_bytes, bar);
    });
}

template <typename S, int PARITY, int FEAT, int NSTAGE>
__global__ void __launch_bounds__(256) k_rows(const StepArgs a, int* error) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t nx = uint32_t(a.nx), ny = uint32_t(a.ny), nz = uint32_t(a.nz);
    const uint32_t nrows = ny * nz;
    const size_t stage_elems = size_t(19) * nx;
    const size_t stage_bytes = (stage_elems * sizeof(S) + 127) / 128 * 128;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + NSTAGE * stage_bytes);
    auto stage = [&](int s) { return reinterpret_cast<S*>(smem_raw + size_t(s) * stage_bytes); };
    const bool leader = threadIdx.x == 0;
    const long long limit = 1ll << 22;  // polls per wait (a copy completes in microseconds)

    if (leader) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // prologue: the first NSTAGE rows of this block
    if (leader)
        for (int s = 0; s < NSTAGE; ++s) {
            const uint32_t row = blockIdx.x + uint32_t(s) * gridDim.x;
            if (row < nrows) issue_row<S, PARITY>(a, row, stage(s), &bars[s]);
        }
    S* __restrict__ f = static_cast<S*>(a.f);
    const uint64_t P = a.plane;
    __shared__ int abort_flag;
    if (leader) abort_flag = 0;
    __syncthreads();

    uint32_t k = 0;
    for (uint32_t row = blockIdx.x; row < nrows; row += gridDim.x, ++k) {
        const int s = int(k % NSTAGE);
        const uint32_t parity = (k / NSTAGE) & 1u;
        // every thread polls the barrier itself (bounded); a failure anywhere aborts the block
        if (!mbar_wait_bounded(&bars[s], parity, limit)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
        const S* buf = stage(s);
        const uint32_t y = row % ny, z = row / ny;
        const uint32_t n0 = row * nx;
        // wrapped neighbour rows of this row, as row indices: y part and z part
        const uint32_t row_y0 = y, row_ym = (y == 0) ? ny - 1 : y - 1,
                       row_yp = (y == ny - 1) ? 0 : y + 1;
        const uint32_t plane_z0 = z * ny, plane_zm = ((z == 0) ? nz - 1 : z - 1) * ny,
                       plane_zp = ((z == nz - 1) ? 0 : z + 1) * ny;
        for (uint32_t x = threadIdx.x; x < nx; x += blockDim.x) {
            float fh[19];
            if constexpr (PARITY == 0) {
                sfor<0, 19>([&](auto I) { fh[I] = smem_ld<S>(buf + size_t(I) * nx + x); });
            } else {
                const uint32_t xm = (x == 0) ? nx - 1 : x - 1;
                const uint32_t xp = (x == nx - 1) ? 0 : x + 1;
                sfor<0, 19>([&](auto I) {
                    constexpr int i = I;
                    const uint32_t sx = dcx(i) > 0 ? xm : (dcx(i) < 0 ? xp : x);
                    fh[i] = smem_ld<S>(buf + size_t(i) * nx + sx);
                });
            }
            const uint32_t n = n0 + x;
            float Fx = 0.f, Fy = 0.f, Fz = 0.f;
            cell_force<FEAT>(a, n, Fx, Fy, Fz);
            float ntx = 0.f, nty = 0.f, ntz = 0.f;
            collide<FEAT>(fh, a, int(x), 0.0f, Fx, Fy, Fz, ntx, nty, ntz);
            if constexpr (PARITY == 0) {
                store_ddf<S>(f + n, fh[0]);
                sfor<1, 19>([&](auto I) { store_ddf<S>(f + uint64_t(opp(I)) * P + n, fh[I]); });
            } else {
                const uint32_t xm = (x == 0) ? nx - 1 : x - 1;
                const uint32_t xp = (x == nx - 1) ? 0 : x + 1;
                store_ddf<S>(f + n, fh[0]);
                sfor<1, 19>([&](auto I) {
                    constexpr int i = I;
                    const uint32_t dx = dcx(i) > 0 ? xp : (dcx(i) < 0 ? xm : x);
                    const uint32_t rb = (dcy(i) > 0 ? row_yp : (dcy(i) < 0 ? row_ym : row_y0)) +
                                        (dcz(i) > 0 ? plane_zp : (dcz(i) < 0 ? plane_zm : plane_z0));
                    store_ddf<S>(f + uint64_t(i) * P + uint64_t(rb) * nx + dx, fh[i]);
                });
            }
        }
        __syncthreads();  // the stage is free again
        if (leader) {
            const uint32_t next = row + uint32_t(NSTAGE) * gridDim.x;
            if (next < nrows) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_row<S, PARITY>(a, next, stage(s), &bars[s]);
            }
        }
    }
    if (abort_flag) {
        if (leader) atomicExch(error, 1);
        // let this block's outstanding copies land before shared memory is released
        for (int s = 0; s < NSTAGE; ++s) {
            const uint32_t kk = k + uint32_t(s);
            const uint32_t row = blockIdx.x + kk * gridDim.x;
            if (row < nrows)
                mbar_wait_bounded(&bars[kk % NSTAGE], (kk / NSTAGE) & 1u, limit);
        }
    }
}

constexpr int kStages = 3;
constexpr size_t kMaxRowsSmem = 200 * 1024;  // largest stage set the variant accepts

template <typename S>
size_t rows_smem(int nx) {
    const size_t stage_bytes = (size_t(19) * nx * sizeof(S) + 127) / 128 * 128;
    return kStages * stage_bytes + kStages * sizeof(uint64_t);
}

template <typename S, int PARITY, int FEAT>
const void* rows_fn() {
    return reinterpret_cast<const void*>(&k_rows<S, PARITY, FEAT, kStages>);
}

template <typename S>
const void* pick(int parity, int feat) {
    if (parity == 0)
        return feat == 2 ? rows_fn<S, 0, 2>() : (feat == 1 ? rows_fn<S, 0, 1>() : rows_fn<S, 0, 0>());
    return feat == 2 ? rows_fn<S, 1, 2>() : (feat == 1 ? rows_fn<S, 1, 1>() : rows_fn<S, 1, 0>());
}

}  // namespace

bool rows_step_supported(int half_storage, int geo, bool probe, int nx, int threads) {
    const size_t es = half_storage ? 2 : 4;
    const size_t smem = half_storage ? rows_smem<__half>(nx) : rows_smem<float>(nx);
    return !geo && !probe && (size_t(nx) * es) % 16 == 0 && smem <= kMaxRowsSmem && threads >= 32 &&
           threads <= 256 && threads % 32 == 0;
}

// Resident blocks per SM of one kernel at one (threads, smem), cached: the
// attribute call and the occupancy query cost host time on every launch. The
// dynamic shared-memory limit of a kernel is raised once to kMaxRowsSmem, so a
// cached entry stays valid whatever size another lattice asked for since.
int rows_blocks_per_sm(const void* fn, int threads, size_t smem, cudaError_t* err) {
    struct Entry { const void* fn; int threads; size_t smem; int per_sm; };
    static thread_local Entry cache[32];
    static thread_local int used = 0;
    static thread_local const void* raised[16];
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
        if (nraised < 16) raised[nraised++] = fn;
    }
    int per_sm = 0;
    *err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    if (*err != cudaSuccess) return 0;
    if (used < 32) cache[used++] = Entry{fn, threads, smem, per_sm};
    return per_sm;
}

cudaError_t launch_rows_step(const StepArgs& a, int half_storage, int parity, int feat,
                             int threads, int sm_count, int* error, cudaStream_t st) {
    const void* fn = half_storage ? pick<__half>(parity, feat) : pick<float>(parity, feat);
    const size_t smem = half_storage ? rows_smem<__half>(a.nx) : rows_smem<float>(a.nx);
    cudaError_t e = cudaSuccess;
    const int per_sm = rows_blocks_per_sm(fn, threads, smem, &e);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint32_t nrows = uint32_t(a.ny) * uint32_t(a.nz);
    uint32_t grid = uint32_t(per_sm) * uint32_t(sm_count);
    if (grid > nrows) grid = nrows;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    void* args[] = {const_cast<StepArgs*>(&a), &error};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace stro
