// FP16-storage step with two x-adjacent cells per thread (periodic lattices).
//
// With binary16 DDFs a one-cell thread keeps only 19 x 2 bytes in flight per
// pass, which leaves the step latency-bound. Here each thread owns the cell
// pair (x, x+1), x even, and moves both cells' DDFs as one 4-byte half2 per
// direction (packed conversions, half the load/store instructions). A warp
// covers 64 consecutive cells of one row.
//
// Even pass: all accesses are aligned half2.
// Odd pass: directions with c_x = 0 stay aligned half2. For c_x = +1 the
// sources are x-1 and x: the thread loads the aligned pair (x, x+1) of the
// source row and takes x-1 from the lane below (shfl.up); lane 0 reads the one
// element left of the warp (wrapping at x = 0) directly. c_x = -1 mirrors this
// with shfl.down and lane 31. Stores are the transpose: each lane writes the
// aligned pair it covers with the value shuffled in from its neighbour, and
// the lane at the warp edge writes the single element that belongs to the
// neighbouring warp's pair. Every slot is still read and written exactly once.
//
// The per-cell arithmetic is the shared collide(), so results are identical to
// the one-cell kernels. Requirements (checked by the host): FP16 storage, no
// walls or solid fractions, nx a multiple of 64, even plane stride.
#include "lbm_cell.cuh"
#include "lbm_launch.h"

namespace stro {

namespace {

__device__ __forceinline__ int wrap_x(int v, int nx) {
    v += (v < 0) ? nx : 0;
    v -= (v >= nx) ? nx : 0;
    return v;
}

template <int FEAT>
__global__ void __launch_bounds__(256, 2) k_pair_even(const StepArgs a) {
    const int x = 2 * int(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = int(blockIdx.y * blockDim.y + threadIdx.y);
    const int z = int(blockIdx.z);
    if (y >= a.ny) return;
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(a.nx) + uint32_t(x);
    __half2* __restrict__ f2 = static_cast<__half2*>(a.f);
    const uint64_t P2 = a.plane / 2;
    const uint32_t n2 = n / 2;
    float A[19], B[19];
    sfor<0, 19>([&](auto I) {
        const float2 v = __half22float2(f2[uint64_t(I) * P2 + n2]);
        A[I] = v.x;
        B[I] = v.y;
    });
    float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
    float FAx = 0.f, FAy = 0.f, FAz = 0.f, FBx = 0.f, FBy = 0.f, FBz = 0.f;
    cell_force<FEAT>(a, n, FAx, FAy, FAz);
    cell_force<FEAT>(a, n + 1, FBx, FBy, FBz);
    collide<FEAT>(A, a, x, 0.0f, FAx, FAy, FAz, ax, ay, az);
    collide<FEAT>(B, a, x + 1, 0.0f, FBx, FBy, FBz, bx, by, bz);
    f2[n2] = __floats2half2_rn(A[0], B[0]);
    sfor<1, 19>([&](auto I) { f2[uint64_t(opp(I)) * P2 + n2] = __floats2half2_rn(A[I], B[I]); });
}

template <int FEAT>
__global__ void __launch_bounds__(256, 2) k_pair_odd(const StepArgs a) {
    const int lane = int(threadIdx.x & 31u);
    const int x = 2 * int(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = int(blockIdx.y * blockDim.y + threadIdx.y);
    const int z = int(blockIdx.z);
    if (y >= a.ny) return;  // whole warps share y: no shuffle loses a lane
    const int nx = a.nx;
    const int xw = x - 2 * lane;              // first cell of this warp
    const int x_left = wrap_x(xw - 1, nx);    // element left of the warp
    const int x_right = wrap_x(xw + 64, nx);  // element right of the warp
    const uint32_t n = (uint32_t(z) * uint32_t(a.ny) + uint32_t(y)) * uint32_t(nx) + uint32_t(x);
    const NbrOffsets nb(x, y, z, nx, a.ny, a.nz);
    __half2* __restrict__ f2 = static_cast<__half2*>(a.f);
    __half* __restrict__ f1 = static_cast<__half*>(a.f);
    const uint64_t P = a.plane;
    const uint64_t P2 = P / 2;
    float A[19], B[19];
    {
        const float2 v = __half22float2(f2[n / 2]);
        A[0] = v.x;
        B[0] = v.y;
    }
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        constexpr int o = opp(i);
        // source row of direction i (y, z shifted by -c_i), same x
        const uint32_t r = uint32_t(int(n) + nb.template off<0, -dcy(i), -dcz(i)>());
        const float2 v = __half22float2(f2[uint64_t(o) * P2 + r / 2]);
        if constexpr (dcx(i) == 0) {
            A[i] = v.x;
            B[i] = v.y;
        } else if constexpr (dcx(i) > 0) {  // sources x-1, x
            B[i] = v.x;
            const float left = __shfl_up_sync(0xffffffffu, v.y, 1);
            A[i] = lane == 0 ? __half2float(f1[uint64_t(o) * P + (r - uint32_t(x) + uint32_t(x_left))])
                             : left;
        } else {  // sources x+1, x+2
            A[i] = v.y;
            const float right = __shfl_down_sync(0xffffffffu, v.x, 1);
            B[i] = lane == 31
                       ? __half2float(f1[uint64_t(o) * P + (r - uint32_t(x) + uint32_t(x_right))])
                       : right;
        }
    });
    float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
    float FAx = 0.f, FAy = 0.f, FAz = 0.f, FBx = 0.f, FBy = 0.f, FBz = 0.f;
    cell_force<FEAT>(a, n, FAx, FAy, FAz);
    cell_force<FEAT>(a, n + 1, FBx, FBy, FBz);
    collide<FEAT>(A, a, x, 0.0f, FAx, FAy, FAz, ax, ay, az);
    collide<FEAT>(B, a, x + 1, 0.0f, FBx, FBy, FBz, bx, by, bz);
    f2[n / 2] = __floats2half2_rn(A[0], B[0]);
    sfor<1, 19>([&](auto I) {
        constexpr int i = I;
        // destination row of direction i (y, z shifted by +c_i), same x
        const uint32_t d = uint32_t(int(n) + nb.template off<0, dcy(i), dcz(i)>());
        const uint64_t base = uint64_t(i) * P;
        if constexpr (dcx(i) == 0) {
            f2[uint64_t(i) * P2 + d / 2] = __floats2half2_rn(A[i], B[i]);
        } else if constexpr (dcx(i) > 0) {  // destinations x+1, x+2
            const float lo = __shfl_up_sync(0xffffffffu, B[i], 1);
            if (lane != 0) {
                f2[uint64_t(i) * P2 + d / 2] = __floats2half2_rn(lo, A[i]);
            } else {
                f1[base + d + 1] = __float2half_rn(A[i]);
            }
            if (lane == 31) f1[base + (d - uint32_t(x) + uint32_t(x_right))] = __float2half_rn(B[i]);
        } else {  // destinations x-1, x
            const float hi = __shfl_down_sync(0xffffffffu, A[i], 1);
            if (lane != 31) {
                f2[uint64_t(i) * P2 + d / 2] = __floats2half2_rn(B[i], hi);
            } else {
                f1[base + d] = __float2half_rn(B[i]);
            }
            if (lane == 0) f1[base + (d - uint32_t(x) + uint32_t(x_left))] = __float2half_rn(A[i]);
        }
    });
}

}  // namespace

bool pair_step_supported(int half_storage, int geo, bool probe, int nx, uint64_t plane,
                         dim3 block) {
    return half_storage && !geo && !probe && nx % 64 == 0 && plane % 2 == 0 && block.x % 32 == 0 &&
           (nx / 2) % int(block.x) == 0 && block.x * block.y <= 256;
}

cudaError_t launch_pair_step(const StepArgs& a, int parity, int feat, dim3 block, cudaStream_t st) {
    const dim3 grid(unsigned(a.nx / 2) / block.x, (unsigned(a.ny) + block.y - 1) / block.y,
                    unsigned(a.nz));
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

}  // namespace stro
