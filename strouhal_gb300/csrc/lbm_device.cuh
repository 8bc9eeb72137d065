// D3Q19 lattice helpers shared by the device kernels.
//
// Velocity order and pairing follow the reference (Kernels.metal:38-47): the
// order is load-bearing because the AA pattern stores direction i into slot
// opp(i) on even steps, and the state layout / digest depend on it.
//   i : 0 | 1 2 | 3 4 | 5 6 | 7 8   | 9 10  | 11 12 | 13 14 | 15 16 | 17 18
//   c : 0 |  ±x |  ±y |  ±z | ±(x+y)| ±(x-y)| ±(x+z)| ±(x-z)| ±(y+z)| ±(y-z)
// All lattice tables are constexpr functions so that fully unrolled code folds
// them into immediates.
#pragma once

#include <cuda_fp16.h>
#include <cstdint>
#include <type_traits>

namespace stro {

__host__ __device__ constexpr int dcx(int i) {
    return (i == 1 || i == 7 || i == 9 || i == 11 || i == 13)    ? 1
           : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1
                                                                  : 0;
}
__host__ __device__ constexpr int dcy(int i) {
    return (i == 3 || i == 7 || i == 10 || i == 15 || i == 17)   ? 1
           : (i == 4 || i == 8 || i == 9 || i == 16 || i == 18) ? -1
                                                                 : 0;
}
__host__ __device__ constexpr int dcz(int i) {
    return (i == 5 || i == 11 || i == 14 || i == 15 || i == 18)  ? 1
           : (i == 6 || i == 12 || i == 13 || i == 16 || i == 17) ? -1
                                                                   : 0;
}
__host__ __device__ constexpr int opp(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }

// Lattice weights as FP32 constants (1/3, 1/18, 1/36 correctly rounded).
__host__ __device__ constexpr float wgt(int i) {
    return i == 0 ? 1.0f / 3.0f : (i < 7 ? 1.0f / 18.0f : 1.0f / 36.0f);
}

// Compile-time loop: f(std::integral_constant<int, I>) for I in [B, E).
template <int B, int E, class F>
__device__ __forceinline__ void sfor(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        sfor<B + 1, E>(f);
    }
}

// c_i . v with the components taken in x, y, z order and zero coefficients
// skipped: equal in value to (float)cx*vx + (float)cy*vy + (float)cz*vz.
template <int I>
__device__ __forceinline__ float cdot(float vx, float vy, float vz) {
    constexpr int a = dcx(I), b = dcy(I), c = dcz(I);
    if constexpr (a != 0) {
        float s = a > 0 ? vx : -vx;
        if constexpr (b != 0) s = b > 0 ? s + vy : s - vy;
        if constexpr (c != 0) s = c > 0 ? s + vz : s - vz;
        return s;
    } else if constexpr (b != 0) {
        float s = b > 0 ? vy : -vy;
        if constexpr (c != 0) s = c > 0 ? s + vz : s - vz;
        return s;
    } else {
        return c > 0 ? vz : -vz;
    }
}

// Storage conversions: FP32, or IEEE binary16 with round-to-nearest-even.
template <typename S> __device__ __forceinline__ float load_ddf(const S* p);
template <> __device__ __forceinline__ float load_ddf<float>(const float* p) { return *p; }
template <> __device__ __forceinline__ float load_ddf<__half>(const __half* p) {
    return __half2float(*p);
}
// Load through L2 only (no L1 allocation): used where another SM may have
// rewritten the slot since this SM last read it, inside one launch.
template <typename S> __device__ __forceinline__ float load_ddf_cg(const S* p);
template <> __device__ __forceinline__ float load_ddf_cg<float>(const float* p) { return __ldcg(p); }
template <> __device__ __forceinline__ float load_ddf_cg<__half>(const __half* p) {
    return __half2float(__ldcg(p));
}
template <typename S, bool CG>
__device__ __forceinline__ float load_slot(const S* p) {
    if constexpr (CG) return load_ddf_cg<S>(p);
    else return load_ddf<S>(p);
}
template <typename S> __device__ __forceinline__ void store_ddf(S* p, float v);
template <> __device__ __forceinline__ void store_ddf<float>(float* p, float v) { *p = v; }
template <> __device__ __forceinline__ void store_ddf<__half>(__half* p, float v) {
    *p = __float2half_rn(v);
}

// Multiplier and shift of an exact unsigned division by d (host side):
// n / d = (n * m) >> (32 + s) with s = ceil(log2 d), m = ceil(2^(32+s) / d),
// for n < 2^32 (the error m d - 2^(32+s) is below d <= 2^s); the 64-bit
// product n * m (m < 2^33) does not overflow for n < 2^31.
inline void division_magic(uint32_t d, uint64_t* m, uint32_t* s) {
    uint32_t sh = 0;
    while ((uint64_t(1) << sh) < d) ++sh;
    const unsigned __int128 num = (unsigned __int128)1 << (32 + sh);
    *m = uint64_t((num + d - 1) / d);
    *s = sh;
}

// Cell byte (even pass): low 3 bits = cell type; bit 3 = partially saturated (eps != 0).
constexpr uint8_t CELL_TYPE_MASK = 0x7u;
constexpr uint8_t CELL_EPS_BIT = 0x8u;
enum : uint8_t { CELL_FLUID = 0, CELL_SOLID = 1, CELL_LID = 2, CELL_INFLOW = 3, CELL_OUTFLOW = 4 };

// Geometry word (odd pass): bits 0..17 = neighbour n + c_i is a wall (bit i-1),
// bit 29 = eps != 0, bit 30 = some wall neighbour moves (lid/inflow/outflow),
// bit 31 = the cell itself is not fluid.
constexpr uint32_t GEO_WALL_BITS = 0x3FFFFu;
constexpr uint32_t GEO_EPS = 1u << 29;
constexpr uint32_t GEO_MOVING = 1u << 30;
constexpr uint32_t GEO_NONFLUID = 1u << 31;

// Everything one step launch needs. Passed by value (kernel parameter space).
struct StepArgs {
    void* f;                  // DDF planes (Store*), plane stride `plane` elements
    uint64_t plane;           // plane stride in elements (>= N, padded)
    uint32_t poff[19];        // i * plane: element offset of plane i (0 when 19 planes do
                              // not fit 2^32 elements; read only by kernels that require it)
    int32_t nx, ny, nz;
    const uint8_t* cell;      // N cell bytes (walls or eps present)
    const uint32_t* geo;      // N geometry words
    const uint32_t* lmask;    // N moving-wall masks (bit i-1), read only where GEO_MOVING
    const float* eps;         // N solid fractions, read only where flagged
    const float* ffield;      // optional force field: 3 planes of N floats
    uint32_t ffield_plane;    // plane stride of ffield (= N)
    float omega, omega_minus; // omega+ and omega-
    float tau0;               // 1 / omega (FP32 division), for cells the sponge leaves alone
    float uin;                // ramped inflow peak / uniform velocity
    float c_smago;            // Smagorinsky Cs^2
    float fx, fy, fz;         // uniform Guo force
    float ulid_x, ulid_y, ulid_z;  // ramped lid velocity
    int32_t inflow_uniform;
    float sponge_x0, sponge_inv_w, sponge_tau;
    int32_t force_on;         // any nonzero uniform force or a force field
    int32_t outflow_pressure; // outflow walls: 0 the reference's sign flip, 1 with the u-terms
    void* f_out;              // one-cell kernels of walled lattices and the block-list
                              // kernels of the split: write the pass here instead of in
                              // place (same layout; every slot a fluid cell owns is
                              // written, the other slots are not)
    // force probe (odd pass only)
    int32_t box_x0, box_x1, box_y0, box_y1;
    double* partials;         // 3 doubles per block
};

// Deterministic block reduction of up to 4 doubles (fixed shuffle tree, then
// warps in index order). All threads of the block must call it.
template <int K>
__device__ __forceinline__ void block_reduce_store(double (&v)[K], double* out) {
    __shared__ double warp_sums[32][K];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const int nwarps = (nthreads + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = v[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0) warp_sums[warp][k] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = lane < nwarps ? warp_sums[lane][k] : 0.0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
            if (lane == 0) out[k] = s;
        }
    }
    __syncthreads();  // warp_sums may be reused by the next call
}

}  // namespace stro
