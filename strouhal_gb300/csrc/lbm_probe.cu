// Field initialisation, moments and fixed-order FP64 reductions.
//
// initField restates Kernels.metal:393-453 (trigonometric values are taken in
// double precision and rounded to FP32, so the initial state does not depend
// on a device math library). momentsEven restates Kernels.metal:359-380. The
// reductions (kinetic energy, dissipation, mass, non-finite count) accumulate
// FP64 per thread in a fixed cell order, reduce each block with a fixed
// shuffle tree and fold the block partials in a second fixed-order pass: the
// result is bitwise reproducible run to run (no atomics).
#include "lbm_device.cuh"
#include "lbm_launch.h"

namespace stro {

namespace {

constexpr int kThreads = 256;

template <typename S>
__device__ __forceinline__ void load_cell(const FieldView& v, uint32_t n, float (&fh)[19]) {
    const S* f = static_cast<const S*>(v.f);
    sfor<0, 19>([&](auto I) { fh[I] = load_ddf<S>(f + uint64_t(I) * v.plane + n); });
}

// Moments of one cell after an even step count, as momentsEven computes them.
__device__ __forceinline__ void cell_moments(const FieldView& v, uint32_t n, const float (&fh)[19],
                                             float& rhom1, float& rho, float& ux, float& uy,
                                             float& uz) {
    rhom1 = fh[0];
    sfor<1, 19>([&](auto I) { rhom1 += fh[I]; });
    float px = fh[1], py = fh[3], pz = fh[5];
    sfor<2, 19>([&](auto I) {
        constexpr int i = I;
        if constexpr (dcx(i) > 0) px += fh[i];
        if constexpr (dcx(i) < 0) px -= fh[i];
    });
    sfor<4, 19>([&](auto I) {
        constexpr int i = I;
        if constexpr (dcy(i) > 0) py += fh[i];
        if constexpr (dcy(i) < 0) py -= fh[i];
    });
    sfor<6, 19>([&](auto I) {
        constexpr int i = I;
        if constexpr (dcz(i) > 0) pz += fh[i];
        if constexpr (dcz(i) < 0) pz -= fh[i];
    });
    float Fx = v.fx, Fy = v.fy, Fz = v.fz;
    if (v.ffield != nullptr) {
        Fx = v.fx + v.ffield[n];
        Fy = v.fy + v.ffield[uint64_t(v.N) + n];
        Fz = v.fz + v.ffield[2ull * v.N + n];
    }
    rho = 1.0f + rhom1;
    ux = (px + 0.5f * Fx) / rho;
    uy = (py + 0.5f * Fy) / rho;
    uz = (pz + 0.5f * Fz) / rho;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_init_field(FieldView v, uint32_t mode, float A,
                                                         float tau) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= v.N) return;
    float ux = 0.f, uy = 0.f, uz = 0.f, sxx = 0.f, sxz = 0.f, syz = 0.f, rhom1 = 0.f;
    const uint32_t x = n % v.nx, t = n / v.nx, y = t % v.ny, z = t / v.ny;
    const float pi = 3.14159265358979323846f;
    auto S_ = [](float a) { return (float)sin((double)a); };
    auto C_ = [](float a) { return (float)cos((double)a); };
    if (mode == 1u) {
        const float kx = 2.0f * pi / (float)v.nx, ky = 2.0f * pi / (float)v.ny;
        const float xa = (float)x + 0.5f, ya = (float)y + 0.5f;
        ux = A * S_(kx * xa) * C_(ky * ya);
        uy = -A * C_(kx * xa) * S_(ky * ya);
        sxx = A * kx * C_(kx * xa) * C_(ky * ya);
        rhom1 = 0.75f * A * A * (C_(2.0f * kx * xa) + C_(2.0f * ky * ya));
    }
    if (mode == 2u) {
        const float kx = 2.0f * pi / (float)v.nx, ky = 2.0f * pi / (float)v.ny,
                    kz = 2.0f * pi / (float)v.nz;
        const float xa = kx * ((float)x + 0.5f), ya = ky * ((float)y + 0.5f),
                    za = kz * ((float)z + 0.5f);
        ux = A * S_(xa) * C_(ya) * C_(za);
        uy = -A * C_(xa) * S_(ya) * C_(za);
        sxx = A * kx * C_(xa) * C_(ya) * C_(za);
        sxz = -0.5f * A * kz * S_(xa) * C_(ya) * S_(za);
        syz = 0.5f * A * kz * C_(xa) * S_(ya) * S_(za);
        rhom1 = 0.1875f * A * A * (C_(2.0f * xa) + C_(2.0f * ya)) * (C_(2.0f * za) + 2.0f);
    }
    const float rho = 1.0f + rhom1;
    const float u2 = ux * ux + uy * uy + uz * uz;
    S* f = static_cast<S*>(v.f);
    sfor<0, 19>([&](auto I) {
        constexpr int i = I;
        const float cu = 3.0f * ((float)dcx(i) * ux + (float)dcy(i) * uy + (float)dcz(i) * uz);
        const float feq = wgt(i) * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
        const float cc = (float)(dcx(i) * dcx(i) - dcy(i) * dcy(i));
        const float scc = sxx * cc + 2.0f * sxz * (float)(dcx(i) * dcz(i)) +
                          2.0f * syz * (float)(dcy(i) * dcz(i));
        const float fneq = -3.0f * wgt(i) * tau * scc;
        store_ddf<S>(f + uint64_t(i) * v.plane + n, feq + fneq);
    });
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_moments(FieldView v, float4* out) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= v.N) return;
    if (v.cell != nullptr && (v.cell[n] & CELL_TYPE_MASK) != CELL_FLUID) {
        out[n] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    float fh[19];
    load_cell<S>(v, n, fh);
    float rhom1, rho, ux, uy, uz;
    cell_moments(v, n, fh, rhom1, rho, ux, uy, uz);
    out[n] = make_float4(ux, uy, uz, rho);
}

// Per cell: |u|^2 (FP32, as the host energy loop forms it) and the viscous
// dissipation 2 nu S:S with S = -(3 omega / (2 rho)) Pi_neq.
template <typename S>
__global__ void __launch_bounds__(kThreads) k_observables(FieldView v, float omega,
                                                          double* partials) {
    double acc[2] = {0.0, 0.0};
    const double nu = (1.0 / (double)omega - 0.5) / 3.0;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < v.N; n += gridDim.x * blockDim.x) {
        if (v.cell != nullptr && (v.cell[n] & CELL_TYPE_MASK) != CELL_FLUID) continue;
        float fh[19];
        load_cell<S>(v, n, fh);
        float rhom1, rho, ux, uy, uz;
        cell_moments(v, n, fh, rhom1, rho, ux, uy, uz);
        const float u2 = ux * ux + uy * uy + uz * uz;
        acc[0] += (double)u2;
        float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
        sfor<1, 19>([&](auto I) {
            constexpr int i = I;
            const float cu = 3.0f * cdot<i>(ux, uy, uz);
            const float feq = wgt(i) * (rhom1 + rho * (cu + 0.5f * cu * cu - 1.5f * u2));
            const float d = fh[i] - feq;
            if constexpr (dcx(i) != 0) pxx += d;
            if constexpr (dcy(i) != 0) pyy += d;
            if constexpr (dcz(i) != 0) pzz += d;
            if constexpr (dcx(i) * dcy(i) > 0) pxy += d;
            if constexpr (dcx(i) * dcy(i) < 0) pxy -= d;
            if constexpr (dcx(i) * dcz(i) > 0) pxz += d;
            if constexpr (dcx(i) * dcz(i) < 0) pxz -= d;
            if constexpr (dcy(i) * dcz(i) > 0) pyz += d;
            if constexpr (dcy(i) * dcz(i) < 0) pyz -= d;
        });
        const double pipi = (double)pxx * pxx + (double)pyy * pyy + (double)pzz * pzz +
                            2.0 * ((double)pxy * pxy + (double)pxz * pxz + (double)pyz * pyz);
        const double s = 1.5 * (double)omega / (double)rho;
        acc[1] += 2.0 * nu * s * s * pipi;
    }
    block_reduce_store<2>(acc, partials + 2u * blockIdx.x);
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_mass(FieldView v, double* partials) {
    double acc[1] = {0.0};
    const S* f = static_cast<const S*>(v.f);
    for (int i = 0; i < 19; ++i)
        for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < v.N;
             n += gridDim.x * blockDim.x)
            acc[0] += (double)load_ddf<S>(f + uint64_t(i) * v.plane + n);
    block_reduce_store<1>(acc, partials + blockIdx.x);
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_nonfinite(FieldView v, double* partials) {
    double acc[1] = {0.0};
    const S* f = static_cast<const S*>(v.f);
    for (int i = 0; i < 19; ++i)
        for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < v.N;
             n += gridDim.x * blockDim.x)
            if (!isfinite(load_ddf<S>(f + uint64_t(i) * v.plane + n))) acc[0] += 1.0;
    block_reduce_store<1>(acc, partials + blockIdx.x);
}

template <int K>
__global__ void __launch_bounds__(kThreads) k_fold(const double* partials, int nblocks,
                                                   double* out) {
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += partials[b * K + k];
    block_reduce_store<K>(acc, out);
}

}  // namespace

int reduction_blocks(uint64_t count) {
    uint64_t b = (count + 1023) / 1024;
    if (b < 1) b = 1;
    if (b > 2048) b = 2048;
    return int(b);
}

cudaError_t launch_fold(const double* partials, int nblocks, int K, double* out, cudaStream_t st) {
    switch (K) {
        case 1: k_fold<1><<<1, kThreads, 0, st>>>(partials, nblocks, out); break;
        case 2: k_fold<2><<<1, kThreads, 0, st>>>(partials, nblocks, out); break;
        case 3: k_fold<3><<<1, kThreads, 0, st>>>(partials, nblocks, out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_init_field(const FieldView& v, int half_storage, uint32_t mode, float amplitude,
                              float tau, cudaStream_t st) {
    const unsigned grid = (v.N + kThreads - 1) / kThreads;
    if (half_storage) k_init_field<__half><<<grid, kThreads, 0, st>>>(v, mode, amplitude, tau);
    else k_init_field<float><<<grid, kThreads, 0, st>>>(v, mode, amplitude, tau);
    return cudaGetLastError();
}

cudaError_t launch_moments(const FieldView& v, int half_storage, float4* out, cudaStream_t st) {
    const unsigned grid = (v.N + kThreads - 1) / kThreads;
    if (half_storage) k_moments<__half><<<grid, kThreads, 0, st>>>(v, out);
    else k_moments<float><<<grid, kThreads, 0, st>>>(v, out);
    return cudaGetLastError();
}

cudaError_t launch_observables(const FieldView& v, int half_storage, float omega,
                               double* partials, double* out, cudaStream_t st) {
    const int nb = reduction_blocks(v.N);
    if (half_storage) k_observables<__half><<<nb, kThreads, 0, st>>>(v, omega, partials);
    else k_observables<float><<<nb, kThreads, 0, st>>>(v, omega, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_fold(partials, nb, 2, out, st);
}

cudaError_t launch_mass(const FieldView& v, int half_storage, double* partials, double* out,
                        cudaStream_t st) {
    const int nb = reduction_blocks(v.N);
    if (half_storage) k_mass<__half><<<nb, kThreads, 0, st>>>(v, partials);
    else k_mass<float><<<nb, kThreads, 0, st>>>(v, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_fold(partials, nb, 1, out, st);
}

cudaError_t launch_nonfinite(const FieldView& v, int half_storage, double* partials, double* out,
                             cudaStream_t st) {
    const int nb = reduction_blocks(v.N);
    if (half_storage) k_nonfinite<__half><<<nb, kThreads, 0, st>>>(v, partials);
    else k_nonfinite<float><<<nb, kThreads, 0, st>>>(v, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_fold(partials, nb, 1, out, st);
}

}  // namespace stro
