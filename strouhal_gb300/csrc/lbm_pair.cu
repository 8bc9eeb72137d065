// FP16-storage step with two x-adjacent cells per thread (periodic lattices).
//
// With binary16 DDFs a one-cell thread keeps only 19 x 2 bytes in flight per
// pass and every load is a 2-byte request; the memory system then delivers
// well below its copy bandwidth however many threads are resident. Here each
// thread owns the cell pair (x, x+1), x even, and moves both cells' DDFs as
// one 4-byte half2 per direction. A warp covers 64 consecutive cells of one
// row.
//
// Registers: only one cell's 19 FP32 values are live at a time. After the
// loads, cell x takes the low halves as FP32 while the high halves (cell
// x+1) are repacked two directions per register (10 registers); cell x's
// results are packed the same way before cell x+1 is collided. This keeps
// the working set near 19 + 10 registers plus the collision's temporaries.
//
// Even pass: all accesses are aligned half2.
// Odd pass: directions with c_x = 0 stay aligned half2. For c_x = +1 the
// sources are x-1 and x: the thread loads the aligned pair (x, x+1) of the
// source row and the aligned pair (x-2, x-1) to its left (wrapping at the row
// start) and keeps one half of each; c_x = -1 mirrors this with (x+2, x+3).
// The second word is the neighbouring thread's own word, so it is served by
// L1 and costs no DRAM traffic. The x-shifted results are stored as two 2-byte
// stores per thread (cell x to x+c_x, cell x+1 to x+1+c_x, wrapping at the
// row ends): wide loads matter for bandwidth, store width does not. No lane
// exchange and no warp-edge special case. Every slot is still written exactly
// once.
//
// The wide kernels (V = 4 or 8 cells per thread, below) reuse this pair code
// with 8- or 16-byte loads.
//
// The per-cell arithmetic is the shared collide(), so results are identical to
// the one-cell kernels of the same arithmetic. Compiled twice like
// lbm_step.cu: STRO_ARITH=0 (stro::exact) and 1 (stro::fused); each copy
// exports one PairLaunchers table. Requirements (checked by the host): FP16
// storage, no walls or solid fractions, nx a multiple of 64, even plane
// stride, 19 planes below 2^32 elements (32-bit element indices), blocks of
// one row (block.y = 1, so y and z come from the block index and the
// neighbour-row offsets are block-uniform), block.x a multiple of 32 dividing
// nx/2, at most 256 threads.
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

__device__ __forceinline__ int wrap_x(int v, int nx) {
    v += (v < 0) ? nx : 0;
    v -= (v >= nx) ? nx : 0;
    return v;
}

// Scheduling fence: the packed values pass through an empty asm statement, so
// the compiler must finish everything that produces `done` before it and may
// start anything that consumes `next` only after it. Without it the two
// cells' collisions are interleaved and both sets of 19 values stay live.
__device__ __forceinline__ void order_cells(__half2 (&done)[10], __half2 (&next)[10]) {
    sfor<0, 10>([&](auto K) {
        uint32_t& d = *reinterpret_cast<uint32_t*>(&done[K]);
        uint32_t& n = *reinterpret_cast<uint32_t*>(&next[K]);
        asm volatile("" : "+r"(d), "+r"(n));
    });
}

template <int FEAT>
__device__ __forceinline__ void collide_cell(float (&fh)[19], const StepArgs& a, int x,
                                             uint32_t n) {
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    cell_force<FEAT>(a, n, Fx, Fy, Fz);
    float ntx = 0.f, nty = 0.f, ntz = 0.f;
    collide<FEAT, STRO_ARITH>(fh, a, x, 0.0f, Fx, Fy, Fz, ntx, nty, ntz);
}

// Collide both cells of the packed pairs v[i] = (cell x, cell x+1). On
// return ao[k] holds cell x's post-collision directions (2k, 2k+1) packed,
// and fh cell x+1's post-collision values.
template <int FEAT>
__device__ __forceinline__ void collide_pair(const __half2 (&v)[19], __half2 (&ao)[10],
                                             float (&fh)[19], const StepArgs& a, int x,
                                             uint32_t n) {
    __half2 bi[10];  // cell x+1's inputs, two directions per register
    sfor<0, 9>([&](auto K) { bi[K] = __halves2half2(__high2half(v[2 * K]), __high2half(v[2 * K + 1])); });
    bi[9] = __halves2half2(__high2half(v[18]), __high2half(v[18]));
    sfor<0, 19>([&](auto I) { fh[I] = __low2float(v[I]); });
    collide_cell<FEAT>(fh, a, x, n);
    sfor<0, 9>([&](auto K) { ao[K] = __floats2half2_rn(fh[2 * K], fh[2 * K + 1]); });
    ao[9] = __floats2half2_rn(fh[18], fh[18]);
    order_cells(ao, bi);
    sfor<0, 19>([&](auto I) {
        fh[I] = (I & 1) ? __high2float(bi[I / 2]) : __low2float(bi[I / 2]);
    });
    collide_cell<FEAT>(fh, a, x + 1, n + 1);
}

// The pointer passes through an empty asm statement: addresses formed from it
// afterwards cannot reuse the ones formed before, so the 19 load addresses
// (two registers each) are not kept alive across the collision for the stores.
template <typename P>
__device__ __forceinline__ void forget(P& p) {
    asm volatile("" : "+l"(p));
}
__device__ __forceinline__ void forget_int(int& v) { asm volatile("" : "+r"(v)); }
__device__ __forceinline__ void forget_u32(uint32_t& v) { asm volatile("" : "+r"(v)); }

// Cell x's post-collision direction i from the packed results.
template <int I>
__device__ __forceinline__ __half out_lo(const __half2 (&ao)[10]) {
    return (I & 1) ? __high2half(ao[I / 2]) : __low2half(ao[I / 2]);
}

template <int FEAT>
__global__ void __launch_bounds__(256, FEAT == 2 ? 2 : 4) k_pair_even(const StepArgs a) {
    const int x = 2 * int(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = int(blockIdx.y);  // one row per block: y and z are block-uniform
    const int z = int(blockIdx.z);
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    // per-thread base pointer plus block-uniform plane offsets (32-bit: 19
    // planes < 2^32 elements). Taking the offsets from the launch constants
    // (StepArgs::poff, as the odd pass does) cut this pass's instructions by 15%
    // but made it 3.6% slower: the constant loads sit ahead of the DDF loads.
    __half2* __restrict__ f2n = static_cast<__half2*>(a.f) + n / 2;
    const uint32_t P2 = uint32_t(a.plane / 2);
    __half2 v[19];
    sfor<0, 19>([&](auto I) { v[I] = f2n[uint32_t(I) * P2]; });
    __half2 ao[10];
    float fh[19];
    collide_pair<FEAT>(v, ao, fh, a, x, n);
    forget(f2n);
    // direction i of both cells goes to slot opp(i)
    sfor<0, 19>([&](auto I) {
        f2n[uint32_t(opp(I)) * P2] = __halves2half2(out_lo<I>(ao), __float2half_rn(fh[I]));
    });
}

// Row indices (z * ny + y) of a row and its neighbour rows. The pair kernel
// has one row per block, so there every value is block-uniform; the wide
// kernels below have one row per warp.
struct PairRows {
    uint32_t ym, y0, yp, zm, z0, zp, ny;
    __device__ __forceinline__ PairRows(const StepArgs& a)
        : PairRows(a, blockIdx.y, blockIdx.z) {}
    __device__ __forceinline__ PairRows(const StepArgs& a, uint32_t y, uint32_t z) {
        ny = uint32_t(a.ny);
        const uint32_t nz = uint32_t(a.nz);
        y0 = y;
        ym = (y == 0) ? ny - 1 : y - 1;
        yp = (y == ny - 1) ? 0 : y + 1;
        z0 = z;
        zm = (z == 0) ? nz - 1 : z - 1;
        zp = (z == nz - 1) ? 0 : z + 1;
    }
    // row of the cell at (y + dy, z + dz)
    template <int DY, int DZ>
    __device__ __forceinline__ uint32_t row() const {
        return (DZ > 0 ? zp : (DZ < 0 ? zm : z0)) * ny + (DY > 0 ? yp : (DY < 0 ? ym : y0));
    }
};

// Odd-pass stores of a cell pair. Addresses are a per-thread base pointer
// (the x part, formed again from x after an opaque asm statement so nothing
// of the gather stays in registers across the collisions) plus a
// block-uniform plane-and-row offset.
// `out` is the state written (StepArgs::f, or f_out for an out-of-place pass).
__device__ __forceinline__ void scatter_pair(const StepArgs& a, void* out, const __half2 (&ao)[10],
                                             const float (&fh)[19], int x, const PairRows& rows) {
    forget_int(x);
    const uint32_t nx = uint32_t(a.nx);
    __half* __restrict__ f1 = static_cast<__half*>(out);
    __half* __restrict__ f1x = f1 + x;                       // both cells, c_x = 0
    // x-shifted destinations of the two cells (periodic in x): x-1 and x+2 wrap
    __half* __restrict__ f1m = f1 + wrap_x(x - 1, int(nx));  // cell x,   c_x = -1
    __half* __restrict__ f1a = f1 + (x + 1);                 // cell x,   c_x = +1
    __half* __restrict__ f1b = f1 + x;                       // cell x+1, c_x = -1
    __half* __restrict__ f1p = f1 + wrap_x(x + 2, int(nx));  // cell x+1, c_x = +1
    *reinterpret_cast<__half2*>(f1x + rows.row<0, 0>() * nx) =
        __halves2half2(out_lo<0>(ao), __float2half_rn(fh[0]));
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        // destination row of direction i (y, z shifted by +c_i)
        const uint32_t R = rows.row<dcy(i), dcz(i)>();
        const __half ah = out_lo<i>(ao);           // cell x, direction i
        const __half bh = __float2half_rn(fh[i]);  // cell x+1, direction i
        const uint32_t w1 = a.poff[i] + R * nx;  // element offset of the row start
        if constexpr (dcx(i) == 0) {
            *reinterpret_cast<__half2*>(f1x + w1) = __halves2half2(ah, bh);
        } else {
            // two 2-byte stores: the warp's stores of one direction fill a
            // contiguous 64-element span between them, no lane exchange
            if constexpr (dcx(i) > 0) {
                f1a[w1] = ah;
                f1p[w1] = bh;
            } else {
                f1m[w1] = ah;
                f1b[w1] = bh;
            }
        }
    });
}

template <int FEAT>
__global__ void __launch_bounds__(256, FEAT == 2 ? 2 : 4) k_pair_odd(const StepArgs a) {
    const int x = 2 * int(blockIdx.x * blockDim.x + threadIdx.x);
    const uint32_t nx = uint32_t(a.nx);
    const PairRows rows(a);
    const __half* __restrict__ f = static_cast<const __half*>(a.f);
    const __half* __restrict__ fx = f + x;
    const __half* __restrict__ fl = f + wrap_x(x - 2, int(nx));  // word (x-2, x-1)
    const __half* __restrict__ fr = f + wrap_x(x + 2, int(nx));  // word (x+2, x+3)
    auto word = [](const __half* p) { return *reinterpret_cast<const __half2*>(p); };
    __half2 v[19];
    v[0] = word(fx + rows.row<0, 0>() * nx);
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        // slot opp(i) of the source row (y, z shifted by -c_i), same x
        const uint32_t w1 = a.poff[o] + rows.row<-dcy(i), -dcz(i)>() * nx;
        const __half2 w = word(fx + w1);
        if constexpr (dcx(i) == 0) {
            v[i] = w;
        } else if constexpr (dcx(i) > 0) {  // sources x-1, x
            v[i] = __halves2half2(__high2half(word(fl + w1)), __low2half(w));
        } else {  // sources x+1, x+2
            v[i] = __halves2half2(__high2half(w), __low2half(word(fr + w1)));
        }
    });
    const uint32_t n = rows.row<0, 0>() * nx + uint32_t(x);
    __half2 ao[10];
    float fh[19];
    collide_pair<FEAT>(v, ao, fh, a, x, n);
    scatter_pair(a, a.f, ao, fh, x, rows);
}

// ------------------------------------------------------------ wide variant
// V cells per thread (V = 4: one 8-byte word per direction; V = 8: one
// 16-byte word), so a warp loads 256 or 512 contiguous bytes of a plane per
// request and each thread keeps 19 * 2V bytes in flight. The cells are then
// collided two at a time with the pair kernel's code (collide_pair) and
// stored as it does (one 4-byte word per direction, or two 2-byte stores for
// x-shifted directions of the odd pass) as soon as each pair is done, which
// frees its input registers. Odd-pass gather: a direction with c_x = +1 needs
// cells x-1 .. x+V-2, i.e. the thread's own word shifted by one half, filled
// from the 4-byte word (x-2, x-1) to its left; c_x = -1 takes the word
// (x+V, x+V+1) to its right. The shift is a funnel shift per 4-byte lane;
// the neighbour words are the adjacent threads' own data, served by L1.
// Blocks are bx threads along x (a multiple of 32 dividing nx / V) by `by`
// rows, so every warp covers 32 V cells of one row.
template <int V> struct WideWord { uint32_t w[V / 2]; };

template <int V>
__device__ __forceinline__ WideWord<V> load_wide(const __half* p) {
    WideWord<V> r;
    if constexpr (V == 4) {
        const uint2 t = *reinterpret_cast<const uint2*>(p);
        r.w[0] = t.x; r.w[1] = t.y;
    } else {
        const uint4 t = *reinterpret_cast<const uint4*>(p);
        r.w[0] = t.x; r.w[1] = t.y; r.w[2] = t.z; r.w[3] = t.w;
    }
    return r;
}

__device__ __forceinline__ __half2 as_half2(uint32_t w) {
    return *reinterpret_cast<const __half2*>(&w);
}

template <int FEAT, int V>
__global__ void __launch_bounds__(256, V == 8 ? 2 : 3) k_wide_even(const StepArgs a) {
    const int x = V * int(blockIdx.x * blockDim.x + threadIdx.x);
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    const uint32_t n = (z * uint32_t(a.ny) + y) * uint32_t(a.nx) + uint32_t(x);
    const __half* __restrict__ fn = static_cast<const __half*>(a.f) + n;
    WideWord<V> W[19];
    sfor<0, 19>([&](auto I) { W[I] = load_wide<V>(fn + a.poff[I]); });
    sfor<0, V / 2>([&](auto J) {
        constexpr int j = J;
        __half2 v[19];
        sfor<0, 19>([&](auto I) { v[I] = as_half2(W[I].w[j]); });
        __half2 ao[10];
        float fh[19];
        collide_pair<FEAT>(v, ao, fh, a, x + 2 * j, n + 2 * j);
        uint32_t m = n + 2 * j;
        forget_u32(m);
        __half* __restrict__ q = static_cast<__half*>(a.f) + m;
        // direction i of both cells goes to slot opp(i)
        sfor<0, 19>([&](auto I) {
            *reinterpret_cast<__half2*>(q + a.poff[opp(I)]) =
                __halves2half2(out_lo<I>(ao), __float2half_rn(fh[I]));
        });
    });
}

template <int FEAT, int V>
__global__ void __launch_bounds__(256, V == 8 ? 2 : 3) k_wide_odd(const StepArgs a) {
    const int x = V * int(blockIdx.x * blockDim.x + threadIdx.x);
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    const uint32_t nx = uint32_t(a.nx);
    const PairRows rows(a, y, z);
    const __half* __restrict__ f = static_cast<const __half*>(a.f);
    const int xl = wrap_x(x - 2, int(nx));  // word (x-2, x-1)
    const int xr = wrap_x(x + V, int(nx));  // word (x+V, x+V+1)
    WideWord<V> W[19];
    W[0] = load_wide<V>(f + rows.row<0, 0>() * nx + uint32_t(x));
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        // slot opp(i) of the source row (y, z shifted by -c_i)
        const __half* __restrict__ src = f + (a.poff[opp(i)] + rows.row<-dcy(i), -dcz(i)>() * nx);
        const WideWord<V> w = load_wide<V>(src + uint32_t(x));
        if constexpr (dcx(i) == 0) {
            W[i] = w;
        } else if constexpr (dcx(i) > 0) {  // sources x-1 .. x+V-2
            const uint32_t l = *reinterpret_cast<const uint32_t*>(src + xl);
            W[i].w[0] = __funnelshift_r(l, w.w[0], 16);
            sfor<1, V / 2>([&](auto K) { W[i].w[K] = __funnelshift_r(w.w[K - 1], w.w[K], 16); });
        } else {  // sources x+1 .. x+V
            const uint32_t r = *reinterpret_cast<const uint32_t*>(src + xr);
            sfor<0, V / 2 - 1>([&](auto K) { W[i].w[K] = __funnelshift_r(w.w[K], w.w[K + 1], 16); });
            W[i].w[V / 2 - 1] = __funnelshift_r(w.w[V / 2 - 1], r, 16);
        }
    });
    const uint32_t n = rows.row<0, 0>() * nx + uint32_t(x);
    sfor<0, V / 2>([&](auto J) {
        constexpr int j = J;
        __half2 v[19];
        sfor<0, 19>([&](auto I) { v[I] = as_half2(W[I].w[j]); });
        __half2 ao[10];
        float fh[19];
        collide_pair<FEAT>(v, ao, fh, a, x + 2 * j, n + 2 * j);
        scatter_pair(a, a.f, ao, fh, x + 2 * j, rows);
    });
}


// ------------------------------------------------------ block-list variant
// The bulk blocks of a walled lattice's bulk / boundary split (every cell
// fluid, no wall neighbour, no solid fraction) in FP16 storage, two
// x-adjacent cells per thread: list entry blockIdx.x names a lattice block of
// bx cells by by rows, covered by bx / 2 by by threads. A bulk cell streams as
// a cell of a periodic lattice does (every neighbour is fluid; y, z and x
// wrap), so gather, collision and scatter are the pair kernel's, with the
// neighbour rows taken per thread (a warp spans 64 / bx rows of the block).
// The x-shifted gather reads the aligned word beside the thread's own, which
// may belong to a neighbouring lattice block of another list: only its half
// inside this block's reach is used, and that slot is written by this thread
// alone, as in the pair kernel. Writes go to StepArgs::f_out when it is set
// (the adjoint's out-of-place recomputation). Requirements (checked by the
// host): nx and bx even, even plane stride, 19 planes below 2^32 elements.
//
// The same launch takes the x-face blocks (entries flagged kListFaceBit;
// blocks whose only walls are velocity-inflow columns at x = 0 / nx - 1): each
// thread computes two cells of the block one after the other with the
// one-cell x-face code (the block's cells in row-major order, thread t taking
// cells t and t + threads, so each round is a contiguous, coalesced half of
// the block). Run in one launch with the bulk blocks, a 128-byte line shared
// by an x-face block and the bulk block beside it is fetched from DRAM once;
// as separate launches each fetched the whole line for its half.
template <int FEAT, bool ODD>
__device__ __forceinline__ void face_block(const StepArgs& a, uint32_t bxi, uint32_t byi,
                                           uint32_t z) {
    const uint32_t bx = 2u * blockDim.x, nt = blockDim.x * blockDim.y;
    const uint32_t tid = threadIdx.x + blockDim.x * threadIdx.y;
#pragma unroll 1
    for (uint32_t c = tid; c < 2u * nt; c += nt) {
        const uint32_t cy = c / bx, cx = c - cy * bx;
        const int x = int(bxi * bx + cx), y = int(byi * blockDim.y + cy);
        if (x >= a.nx || y >= a.ny) continue;
        if constexpr (ODD)
            odd_cell_xface<__half, FEAT, STRO_ARITH, true>(a, WallVel(a), x, y, int(z));
        else
            even_cell<__half, 2, FEAT, false, false, STRO_ARITH, true, true>(a, x, y, int(z));
    }
}

// Cell pair (x, x + 1) of this thread in bulk block (bxi, byi, z).
__device__ __forceinline__ void pair_list_cell(uint32_t bxi, uint32_t byi, int& x, uint32_t& y) {
    x = int(2u * (bxi * blockDim.x + threadIdx.x));
    y = byi * blockDim.y + threadIdx.y;
}

template <int FEAT>
__global__ void __launch_bounds__(256, FEAT == 2 ? 3 : 4)
    k_pair_list_even(const StepArgs a, const uint32_t* list, const ListGrid g) {
    const uint32_t e = list[blockIdx.x];
    uint32_t bxi, byi, z;
    block_coords(e & ~kListFaceBit, g, bxi, byi, z);
    if (e & kListFaceBit) {
        face_block<FEAT, false>(a, bxi, byi, z);
        return;
    }
    int x;
    uint32_t y;
    pair_list_cell(bxi, byi, x, y);
    if (x >= a.nx || y >= uint32_t(a.ny) || z >= uint32_t(a.nz)) return;
    const uint32_t n = (z * uint32_t(a.ny) + y) * uint32_t(a.nx) + uint32_t(x);
    const __half* __restrict__ fn = static_cast<const __half*>(a.f) + n;
    __half2 v[19];
    sfor<0, 19>([&](auto I) { v[I] = *reinterpret_cast<const __half2*>(fn + a.poff[I]); });
    __half2 ao[10];
    float fh[19];
    collide_pair<FEAT>(v, ao, fh, a, x, n);
    uint32_t m = n;
    forget_u32(m);
    __half* __restrict__ q = static_cast<__half*>(a.f_out != nullptr ? a.f_out : a.f) + m;
    // direction i of both cells goes to slot opp(i)
    sfor<0, 19>([&](auto I) {
        *reinterpret_cast<__half2*>(q + a.poff[opp(I)]) =
            __halves2half2(out_lo<I>(ao), __float2half_rn(fh[I]));
    });
}

template <int FEAT>
__global__ void __launch_bounds__(256, FEAT == 2 ? 3 : 4)
    k_pair_list_odd(const StepArgs a, const uint32_t* list, const ListGrid g) {
    const uint32_t e = list[blockIdx.x];
    uint32_t bxi, byi, z;
    block_coords(e & ~kListFaceBit, g, bxi, byi, z);
    if (e & kListFaceBit) {
        face_block<FEAT, true>(a, bxi, byi, z);
        return;
    }
    int x;
    uint32_t y;
    pair_list_cell(bxi, byi, x, y);
    if (x >= a.nx || y >= uint32_t(a.ny) || z >= uint32_t(a.nz)) return;
    const uint32_t nx = uint32_t(a.nx);
    const PairRows rows(a, y, z);
    const __half* __restrict__ f = static_cast<const __half*>(a.f);
    const __half* __restrict__ fx = f + x;
    const __half* __restrict__ fl = f + wrap_x(x - 2, int(nx));  // word (x-2, x-1)
    const __half* __restrict__ fr = f + wrap_x(x + 2, int(nx));  // word (x+2, x+3)
    auto word = [](const __half* p) { return *reinterpret_cast<const __half2*>(p); };
    __half2 v[19];
    v[0] = word(fx + rows.row<0, 0>() * nx);
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        // slot opp(i) of the source row (y, z shifted by -c_i), same x
        const uint32_t w1 = a.poff[o] + rows.row<-dcy(i), -dcz(i)>() * nx;
        const __half2 w = word(fx + w1);
        if constexpr (dcx(i) == 0) {
            v[i] = w;
        } else if constexpr (dcx(i) > 0) {  // sources x-1, x
            v[i] = __halves2half2(__high2half(word(fl + w1)), __low2half(w));
        } else {  // sources x+1, x+2
            v[i] = __halves2half2(__high2half(w), __low2half(word(fr + w1)));
        }
    });
    const uint32_t n = rows.row<0, 0>() * nx + uint32_t(x);
    __half2 ao[10];
    float fh[19];
    collide_pair<FEAT>(v, ao, fh, a, x, n);
    scatter_pair(a, a.f_out != nullptr ? a.f_out : a.f, ao, fh, x, rows);
}

}  // namespace

bool pair_step_supported(int half_storage, int geo, bool probe, int nx, uint64_t plane,
                         dim3 block) {
    return half_storage && !geo && !probe && nx % 64 == 0 && plane % 2 == 0 && block.x % 32 == 0 &&
           (nx / 2) % int(block.x) == 0 && block.y == 1 && block.x <= 256 &&
           19 * plane < (uint64_t(1) << 32);  // element indices fit 32 bits
}

cudaError_t launch_pair_step(const StepArgs& a, int parity, int feat, dim3 block, cudaStream_t st) {
    const dim3 grid(unsigned(a.nx / 2) / block.x, unsigned(a.ny), unsigned(a.nz));
    if (parity == 0) {
        if (feat == 2) k_pair_even<2><<<grid, block, 0, st>>>(a);
        else if (feat == 1) k_pair_even<1><<<grid, block, 0, st>>>(a);
        else k_pair_even<0><<<grid, block, 0, st>>>(a);
    } else {
        if (feat == 2) k_pair_odd<2><<<grid, block, 0, st>>>(a);
        else if (feat == 1) k_pair_odd<1><<<grid, block, 0, st>>>(a);
        else k_pair_odd<0><<<grid, block, 0, st>>>(a);
    }
    return cudaGetLastError();
}

bool wide_step_supported(int half_storage, int geo, bool probe, int nx, int ny, uint64_t plane,
                         dim3 block, int cells) {
    return half_storage && !geo && !probe && (cells == 4 || cells == 8) &&
           nx % (32 * cells) == 0 && plane % 8 == 0 && block.x % 32 == 0 &&
           (nx / cells) % int(block.x) == 0 && block.y >= 1 && ny % int(block.y) == 0 &&
           block.x * block.y <= 256 && 19 * plane < (uint64_t(1) << 32);
}

template <int V>
static void launch_wide_cells(const StepArgs& a, int parity, int feat, dim3 block,
                              cudaStream_t st) {
    const dim3 grid(unsigned(a.nx / V) / block.x, unsigned(a.ny) / block.y, unsigned(a.nz));
    if (parity == 0) {
        if (feat == 2) k_wide_even<2, V><<<grid, block, 0, st>>>(a);
        else if (feat == 1) k_wide_even<1, V><<<grid, block, 0, st>>>(a);
        else k_wide_even<0, V><<<grid, block, 0, st>>>(a);
    } else {
        if (feat == 2) k_wide_odd<2, V><<<grid, block, 0, st>>>(a);
        else if (feat == 1) k_wide_odd<1, V><<<grid, block, 0, st>>>(a);
        else k_wide_odd<0, V><<<grid, block, 0, st>>>(a);
    }
}

cudaError_t launch_wide_step(const StepArgs& a, int parity, int feat, dim3 block, int cells,
                             cudaStream_t st) {
    if (cells == 8) launch_wide_cells<8>(a, parity, feat, block, st);
    else launch_wide_cells<4>(a, parity, feat, block, st);
    return cudaGetLastError();
}

bool pair_list_supported(int half_storage, int feat, int nx, uint64_t plane, dim3 block) {
    return half_storage && feat >= 0 && feat <= 2 && nx % 2 == 0 && block.x % 2 == 0 &&
           (block.x / 2) * block.y <= 256 && plane % 2 == 0 &&
           19 * plane < (uint64_t(1) << 32);  // element indices fit 32 bits
}

cudaError_t launch_pair_list(const StepArgs& a, int parity, int feat, dim3 block,
                             const uint32_t* list, uint32_t count, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const ListGrid g = list_grid(a, block);
    const dim3 threads(block.x / 2, block.y);
    if (parity == 0) {
        if (feat == 2) k_pair_list_even<2><<<count, threads, 0, st>>>(a, list, g);
        else if (feat == 1) k_pair_list_even<1><<<count, threads, 0, st>>>(a, list, g);
        else k_pair_list_even<0><<<count, threads, 0, st>>>(a, list, g);
    } else {
        if (feat == 2) k_pair_list_odd<2><<<count, threads, 0, st>>>(a, list, g);
        else if (feat == 1) k_pair_list_odd<1><<<count, threads, 0, st>>>(a, list, g);
        else k_pair_list_odd<0><<<count, threads, 0, st>>>(a, list, g);
    }
    return cudaGetLastError();
}

const PairLaunchers kPair = {&pair_step_supported, &launch_pair_step, &wide_step_supported,
                             &launch_wide_step, &pair_list_supported, &launch_pair_list};

}  // namespace STRO_ARITH_NS
}  // namespace stro
